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
  double dx, dy, inv_dx, inv_dy, inv_4dx, inv_4dy;
  double cs, dfloor, nu, smag_c, drag;
  double g0, g1, beta, delta;
  int has_delta, blend, floor_v, floor_out, want_cfl, visc_on, smag_on, drag_on, trace_on;
};

// Launchers defined in stage_<recon>.cu.
typedef cudaError_t (*StageLauncher)(int dtype, int rsolver, const StageParams& p, dim3 grid,
                                     size_t smem, cudaStream_t s);
cudaError_t launch_stage_dc(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_stage_plm(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_stage_ppm4(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_stage_ppmx(int, int, const StageParams&, dim3, size_t, cudaStream_t);
cudaError_t launch_stage_wenoz(int, int, const StageParams&, dim3, size_t, cudaStream_t);

typedef cudaError_t (*FaceStatesLauncher)(int dtype, const void* W, int ny, int nx, int nv,
                                          int axis, double dfloor, void* left, void* right,
                                          cudaStream_t s);
cudaError_t face_states_dc(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);
cudaError_t face_states_plm(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);
cudaError_t face_states_ppm4(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);
cudaError_t face_states_ppmx(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);
cudaError_t face_states_wenoz(int, const void*, int, int, int, int, double, void*, void*, cudaStream_t);

// Shared-memory bytes of one stage tile.
inline size_t stage_smem_bytes(int recon, int dtype, int nv, int tx, int ty) {
  int h = recon == JX_DC ? 1 : (recon == JX_PLM ? 2 : 3);
  size_t w = dtype == JX_F64 ? 8 : 4;
  size_t cells = (size_t)nv * ((size_t)(tx + 2 * h) * (ty + 2 * h) +
                               2 * (size_t)ty * (tx + 1) + 2 * (size_t)(ty + 1) * tx);
  return cells * w;
}

}  // namespace jx
