// Parameter blocks and launch helpers for the kernels in jx_aux.cu.
#pragma once
#include "jx_device.cuh"
#include "jx_internal.h"

namespace jx {

struct DtParams {
  double dx, dy, nu, smag_cs, smag_c, drag;
};

struct BeginParams {
  DtParams q;
  jx_clock* clock;
  const double* partials;
  const WsHeader* header;
  int forced, pad;
};

struct CflParams {
  const void* X;  // U (conserved) or W (primitives)
  const jx_clock* clock;  // may be null
  double* partials;
  WsHeader* header;
  int ny, nx, nv, smag;
  double cs, dfloor, inv_dx, inv_dy, inv_4dx, inv_4dy;
};

struct RenderParams {
  const jx_clock* clock;
  const double* table;
  const void *cos_x, *sin_x, *cos_y, *sin_y;
  void* raw;
  int ny, nx, n_modes, n_updates;
};

struct ForceParams {
  const jx_clock* clock;
  const void* U;   // state read by the sums
  void* Uw;        // state written by the kick (same buffer)
  const void* raw;
  double* p1;      // normalisation-moment partials (8 per block)
  double* scal;    // mean_x, mean_y, scale, m0, m1
  double* partials;  // CFL partials
  WsHeader* header;
  void *before_kick, *acceleration, *conserved;  // trace outputs or null
  int ny, nx, nv, nblk, want_cfl;
  int64_t chunk;
  double dfloor, cs;
};

cudaError_t launch_begin_step(const DtParams& q, jx_clock* clock, const double* partials,
                              const WsHeader* hdr, int forced, cudaStream_t s);
cudaError_t launch_begin_step_batch(const BeginParams* solves, int n, cudaStream_t s);
cudaError_t launch_timestep_finish(const DtParams& q, const double* partials, const WsHeader* hdr,
                                   double prev_dt, double time, double tlim, double cfl,
                                   double* dt_out, cudaStream_t s);
int cfl_grid(int64_t ncell);
cudaError_t launch_cfl(int dtype, bool from_w, const CflParams& q, cudaStream_t s);
cudaError_t launch_render(int dtype, const RenderParams& q, cudaStream_t s);
void force_decomposition(int64_t ncell, int* nblk, int64_t* chunk);
cudaError_t launch_force_kick(int dtype, const ForceParams& q, cudaStream_t s);
// Batched forcing over n solves of one precision: render blocks, pass-1/2
// blocks (force_decomposition's nblk) and kick blocks (kick_blocks) per solve
// are laid end to end; off[i] is solve i's first block, off[n] the total.
int render_blocks(int ny, int nx);
// Kick grid: kKickCellsPerBlock cells per block (8 per thread), at most
// kCflBlocksMax blocks (the CFL partial slots).
constexpr int kKickCellsPerBlock = 8 * kReduceThreads;
int kick_blocks(int64_t ncell);
cudaError_t launch_render_batch(int dtype, const RenderParams* q, const int* off, int n, int nwork, cudaStream_t s);
cudaError_t launch_force_kick_batch(int dtype, const ForceParams* q, int n, const int* off_sum, int sum_work,
                                    const int* off_kick, int kick_work, cudaStream_t s);
cudaError_t launch_recover(int dtype, const void* U, void* Uo, void* W, int64_t ncell, int nv,
                           double dfloor, cudaStream_t s);
cudaError_t launch_rk_stage(int dtype, int64_t n, const void* U, const void* V, const void* D,
                            void* Uo, void* Vo, double dt, double g0, double g1, double beta,
                            double delta, int has_delta, int blend, cudaStream_t s);
cudaError_t launch_divergence(int dtype, int ny, int nx, int nv, const void* Fx, const void* Fy,
                              double inv_dx, double inv_dy, void* D, cudaStream_t s);
cudaError_t launch_stress_faces(int dtype, int ny, int nx, const void* tau, void* Fx, void* Fy,
                                cudaStream_t s);
cudaError_t launch_box_sums(int dtype, const void* U, int64_t ncell, int nv, double* part,
                            double* out, cudaStream_t s);
cudaError_t launch_face_flux(int dtype, int rsolver, int64_t nface, int nv, int axis, const void* L,
                             const void* Rr, double cs, void* F, cudaStream_t s);
cudaError_t launch_viscous_flux(int dtype, int ny, int nx, int nv, const void* W, double dx, double dy,
                                double nu, double smag_cs, int axis, void* out, cudaStream_t s);
cudaError_t launch_probe(int dtype, int blocks, int iters, int chains, double* sink, cudaStream_t s);
cudaError_t launch_face_gradients(int dtype, int ny, int nx, int nv, const void* W, double dx, double dy, int axis,
                                  void* gx, void* gy, cudaStream_t s);
cudaError_t launch_smagorinsky(int dtype, int64_t n, const void* gx, const void* gy, double c, void* out,
                               cudaStream_t s);
cudaError_t launch_math_probe(int dtype, int64_t n, const void* a, const void* b, void* rcp_out, void* div_out,
                              void* geo_out, cudaStream_t s);

}  // namespace jx
