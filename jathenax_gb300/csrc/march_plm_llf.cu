// Register-marching stage-kernel instantiations for the plm reconstruction
// with the llf Riemann solver (float64 and float32, 3 or 4 variables).
#include "jx_stage_march.cuh"

namespace jx {
cudaError_t launch_march_plm_llf(int dtype, const StageParams& p, dim3 grid, cudaStream_t s) {
  return launch_march_rs<JX_PLM, JX_LLF>(dtype, p, grid, s);
}
cudaError_t launch_batch_march_plm_llf(int dtype, int nv, int nc, int ring, int form, const StageParams* params, const int* offsets,
                                  int nsolves, int nwork, dim3 grid, cudaStream_t s) {
  return launch_batch_march_rs<JX_PLM, JX_LLF>(dtype, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
}
int march_blocks_per_sm_plm_llf(int dtype, int nv, int nc, int kind) {
  return march_blocks_per_sm_rs_dtype<JX_PLM, JX_LLF>(dtype, nv, nc, kind);
}
}  // namespace jx
