// Launch parameter blocks shared by the C-ABI layer (jx_api.cu) and the
// kernels. Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/jx.h"

namespace jx {

constexpr int kStageThreads = 256;
// Workspace layout (bytes): [header 256][cfl partials][force partials]...
constexpr size_t kWsHeader = 256;
constexpr int kCflSlots = 4;          // per block: max(|vx|+cs), max(|vy|+cs), max strain^2, spare
constexpr int kReduceThreads = 256;   // aux reductions
constexpr int kForceBlocksMax = 512;  // fixed decomposition for forcing / box sums
constexpr int kCflBlocksMax = 2048;   // grid of the standalone CFL and kick kernels

struct WsHeader {
  int64_t n_cfl;  // number of valid CFL partial slots (written by the producer)
  int64_t pad[31];
};

// Loop-invariant constants of one stage, precomputed on the host in the
// state's precision (no per-thread float64 work in the float32 kernel).
template <typename R> struct StageConsts {
  R cs, cs2, inv_cs, half_inv_cs;
  R inv_dx, inv_dy, inv_4dx, inv_4dy;
  R dfloor, nu, smag_c, drag;
  R g0, g1, delta;
};

struct StageParams {
  const void* U;      // stage input, read with halo
  const void* V;      // saved register, pointwise
  void* Uout;         // stage output, pointwise
  void* Vout;         // saved register output (RK4 delta stages) or null
  const void* tau;    // SGS stress (ny, nx, 3) or null
  const jx_clock* clock;
  double* partials;   // CFL partial slots (kCflSlots per block)
  WsHeader* header;
  jx_trace trace;
  int ny, nx, nv, tx, ty, tiles_x;
  int nc;  // marching kernel: columns per lane (tx = 32 nc - 6)
  double dx, dy, inv_dx, inv_dy, inv_4dx, inv_4dy;
  double cs, dfloor, nu, smag_c, drag;
  double g0, g1, beta, delta;
  StageConsts<double> cd;
  StageConsts<float> cf;
  int has_delta, blend, floor_v, floor_out, want_cfl, visc_on, smag_on, drag_on, trace_on;
  int skip;  // batch only: this solve has no such stage
};

template <typename R> __host__ __device__ inline const StageConsts<R>& stage_consts(const StageParams& p);
template <> __host__ __device__ inline const StageConsts<double>& stage_consts<double>(const StageParams& p) { return p.cd; }
template <> __host__ __device__ inline const StageConsts<float>& stage_consts<float>(const StageParams& p) { return p.cf; }

template <typename R>
inline void fill_stage_consts(StageConsts<R>& c, const StageParams& p) {
  c.cs = (R)p.cs;
  c.cs2 = (R)(p.cs * p.cs);
  c.inv_cs = (R)(1.0 / p.cs);
  c.half_inv_cs = (R)(0.5 / p.cs);
  c.inv_dx = (R)p.inv_dx;
  c.inv_dy = (R)p.inv_dy;
  c.inv_4dx = (R)p.inv_4dx;
  c.inv_4dy = (R)p.inv_4dy;
  c.dfloor = (R)p.dfloor;
  c.nu = (R)p.nu;
  c.smag_c = (R)p.smag_c;
  c.drag = (R)p.drag;
  c.g0 = (R)p.g0;
  c.g1 = (R)p.g1;
  c.delta = (R)p.delta;
}

// Launchers defined in stage_<recon>.cu.
typedef cudaError_t (*StageLauncher)(int dtype, int rsolver, const StageParams& p, dim3 grid,
                                     size_t smem, cudaStream_t s);
cudaError_t launch_stage_dc(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_stage_plm(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_stage_ppm4(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_stage_ppmx(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_stage_wenoz(int, int, const StageParams&, dim3, size_t, cudaStream_t);

cudaError_t launch_fast_dc(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_fast_plm(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_fast_ppm4(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_fast_ppmx(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_fast_wenoz(int, int, const StageParams&, dim3, size_t, cudaStream_t);

cudaError_t launch_batch_dc(int, int, const StageParams*, const int*, int, int, dim3, size_t, cudaStream_t);
cudaError_t launch_batch_plm(int, int, const StageParams*, const int*, int, int, dim3, size_t, cudaStream_t);
cudaError_t launch_batch_ppm4(int, int, const StageParams*, const int*, int, int, dim3, size_t, cudaStream_t);
cudaError_t launch_batch_ppmx(int, int, const StageParams*, const int*, int, int, dim3, size_t, cudaStream_t);
cudaError_t launch_batch_wenoz(int, int, const StageParams*, const int*, int, int, dim3, size_t, cudaStream_t);
int batch_blocks_per_sm_dc(int dtype, int rsolver, size_t smem);
int batch_blocks_per_sm_plm(int dtype, int rsolver, size_t smem);
int batch_blocks_per_sm_ppm4(int dtype, int rsolver, size_t smem);
int batch_blocks_per_sm_ppmx(int dtype, int rsolver, size_t smem);
int batch_blocks_per_sm_wenoz(int dtype, int rsolver, size_t smem);

// Shared memory of the 3/4-variable fast stage kernel (tile width 32): the
// same planes as the generic kernel, stored as 4-wide cell vectors.
inline size_t fast_smem_bytes(int recon, int dtype, int ty) {
  const int h = recon == JX_DC ? 1 : (recon == JX_PLM ? 2 : 3);
  const size_t tx = 32;
  const size_t w = (tx + 2 * h) * (size_t)(ty + 2 * h), fx = (size_t)ty * (tx + 1), fy = (size_t)(ty + 1) * tx;
  const size_t ax = (size_t)ty * (tx + 3), ay = (size_t)(ty + 3) * tx;
  const size_t a = (recon == JX_PPM4 || recon == JX_PPMX) ? (ax > ay ? ax : ay) : 0;
  const size_t r = fx > fy ? fx : fy;
  return (w + fx + fy + a + r) * 4 * (dtype == JX_F64 ? 8 : 4);
}

// Register-marching stage kernel (jx_stage_march.cuh): one warp per tile of
// march_tile_x(nc) columns by StageParams::ty rows (nc = 1, 2 or 3 columns
// per lane, 3 ghost columns per side of the 32 nc-column strip); the default
// is two columns (58-column tiles). Blocks are single warps: the warps share
// nothing, and the SM's register file then holds as many warps as registers
// allow (no rounding to whole multi-warp blocks).
constexpr int kMarchWarps = 1;
__host__ __device__ constexpr int march_tile_x(int nc) { return 32 * nc - 6; }
constexpr int kMarchTileX = march_tile_x(2);
constexpr int kMarchMinRows = 8;
// Float32 marching kernels stage a tile's rows in a shared-memory ring (see
// jx_stage_march.cuh) on tiles of at least kRingMinRows rows, for the
// reconstructions and column counts where that measured faster: not DC, and
// WENO-Z with one column per lane only.
constexpr int kRingMinRows = 24;
__host__ __device__ constexpr bool march_ring_built(bool f32, int recon, int nc) {
  return f32 && recon != JX_DC && (recon != JX_WENOZ || nc == 1);
}
// Which marching kernel an occupancy query is for.
enum MarchKind {
  kMarchSingle = 0,
  kMarchSingleLean = 1,
  kMarchBatch = 2,
  kMarchBatchRing = 3,
  kMarchBatchPacked = 4,      // a lean 4-variable group: the packed walk where it is used
  kMarchBatchPackedRing = 5
};
// Compile-time form of a marching launch. kMarchGeneric reads every stage
// option from StageParams at run time; the two lean forms are the stages of
// a problem without viscosity, SGS stress or drag (the inviscid runs) with
// the RK combine's blend form fixed, so that the walk carries no viscous
// window row and tests no per-launch flag in its steady state.
enum MarchForm { kMarchGeneric = 0, kMarchLeanPlain = 1, kMarchLeanBlend = 2 };
// Columns per lane of a marching tile width (0: not a marching width).
inline int march_cols(int tile_x) {
  for (int nc = 1; nc <= 3; ++nc)
    if (tile_x == march_tile_x(nc)) return nc;
  return 0;
}

cudaError_t launch_march_dc(int, int, const StageParams&, dim3, cudaStream_t);
cudaError_t launch_march_plm(int, int, const StageParams&, dim3, cudaStream_t);
cudaError_t launch_march_ppm4(int, int, const StageParams&, dim3, cudaStream_t);
cudaError_t launch_march_ppmx(int, int, const StageParams&, dim3, cudaStream_t);
cudaError_t launch_march_wenoz(int, int, const StageParams&, dim3, cudaStream_t);
// (dtype, rsolver, nv, nc, params, tile offsets, nsolves, nwork, grid, stream)
cudaError_t launch_batch_march_dc(int, int, int, int, int, int, const StageParams*, const int*, int, int, dim3, cudaStream_t);
cudaError_t launch_batch_march_plm(int, int, int, int, int, int, const StageParams*, const int*, int, int, dim3, cudaStream_t);
cudaError_t launch_batch_march_ppm4(int, int, int, int, int, int, const StageParams*, const int*, int, int, dim3, cudaStream_t);
cudaError_t launch_batch_march_ppmx(int, int, int, int, int, int, const StageParams*, const int*, int, int, dim3, cudaStream_t);
cudaError_t launch_batch_march_wenoz(int, int, int, int, int, int, const StageParams*, const int*, int, int, dim3, cudaStream_t);
int march_blocks_per_sm_dc(int dtype, int rsolver, int nv, int nc, int kind);
int march_blocks_per_sm_plm(int dtype, int rsolver, int nv, int nc, int kind);
int march_blocks_per_sm_ppm4(int dtype, int rsolver, int nv, int nc, int kind);
int march_blocks_per_sm_ppmx(int dtype, int rsolver, int nv, int nc, int kind);
int march_blocks_per_sm_wenoz(int dtype, int rsolver, int nv, int nc, int kind);

typedef cudaError_t (*FaceStatesLauncher)(int dtype, const void* W, int ny, int nx, int nv,
                                          int axis, double dfloor, void* left, void* right,
                                          cudaStream_t s);
cudaError_t face_states_dc(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);
cudaError_t face_states_plm(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);
cudaError_t face_states_ppm4(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);
cudaError_t face_states_ppmx(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);
cudaError_t face_states_wenoz(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);

// Shared-memory planes of one stage tile, per variable: primitives with
// halo, x fluxes, y fluxes, face values (PPM4/PPMX), right face states.
struct TilePlanes {
  int halo, pw, ph, w, fx, fy, a, r;
  __host__ __device__ size_t per_var() const { return (size_t)w + fx + fy + a + r; }
};

__host__ __device__ inline TilePlanes tile_planes(int recon, int tx, int ty) {
  TilePlanes t;
  t.halo = recon == JX_DC ? 1 : (recon == JX_PLM ? 2 : 3);
  t.pw = tx + 2 * t.halo;
  t.ph = ty + 2 * t.halo;
  t.w = t.pw * t.ph;
  t.fx = ty * (tx + 1);
  t.fy = (ty + 1) * tx;
  const bool shared = recon == JX_PPM4 || recon == JX_PPMX;
  const int ax = ty * (tx + 3), ay = (ty + 3) * tx;
  t.a = shared ? (ax > ay ? ax : ay) : 0;
  t.r = t.fx > t.fy ? t.fx : t.fy;
  return t;
}

inline size_t stage_smem_bytes(int recon, int dtype, int nv, int tx, int ty) {
  return (size_t)nv * tile_planes(recon, tx, ty).per_var() * (dtype == JX_F64 ? 8 : 4);
}

}  // namespace jx
