// Register-marching stage-kernel instantiations for the ppmx reconstruction
// (float64 and float32, all three Riemann solvers, 3 or 4 variables).
#include "jx_stage_march.cuh"

namespace jx {
cudaError_t launch_march_ppmx(int dtype, int rsolver, const StageParams& p, dim3 grid, cudaStream_t s) {
  return launch_march_recon<JX_PPMX>(dtype, rsolver, p, grid, s);
}
cudaError_t launch_batch_march_ppmx(int dtype, int rsolver, int nv, int nc, const StageParams* params, const int* offsets,
                                  int nsolves, int nwork, dim3 grid, cudaStream_t s) {
  return launch_batch_march_recon<JX_PPMX>(dtype, rsolver, nv, nc, params, offsets, nsolves, nwork, grid, s);
}
int march_blocks_per_sm_ppmx(int dtype, int rsolver, int nv, int nc, bool batch) {
  return march_blocks_per_sm_recon<JX_PPMX>(dtype, rsolver, nv, nc, batch);
}
}  // namespace jx
