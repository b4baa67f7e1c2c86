// Stage-kernel instantiations (generic and 3/4-variable fast path) for the wenoz reconstruction (float64 and
// float32, all three Riemann solvers). One file per reconstruction keeps
// the per-file compile short and lets the build run them in parallel.
#include "jx_stage.cuh"
#include "jx_stage_fast.cuh"

namespace jx {
cudaError_t launch_stage_wenoz(int dtype, int rsolver, const StageParams& p, dim3 grid, size_t smem,
                            cudaStream_t s) {
  return launch_stage_recon<JX_WENOZ>(dtype, rsolver, p, grid, smem, s);
}
cudaError_t face_states_wenoz(int dtype, const void* W, int ny, int nx, int nv, int axis, double dfloor,
                           void* left, void* right, cudaStream_t s) {
  return launch_face_states_recon<JX_WENOZ>(dtype, W, ny, nx, nv, axis, dfloor, left, right, s);
}
cudaError_t launch_fast_wenoz(int dtype, int rsolver, const StageParams& p, dim3 grid, size_t smem,
                           cudaStream_t s) {
  return launch_fast_recon<JX_WENOZ>(dtype, rsolver, p, grid, smem, s);
}
cudaError_t launch_batch_wenoz(int dtype, int rsolver, const StageParams* params, const int* offsets, int nsolves,
                            int nwork, dim3 grid, size_t smem, cudaStream_t s) {
  return launch_batch_recon<JX_WENOZ>(dtype, rsolver, params, offsets, nsolves, nwork, grid, smem, s);
}
int batch_blocks_per_sm_wenoz(int dtype, int rsolver, size_t smem) {
  return batch_blocks_per_sm_recon<JX_WENOZ>(dtype, rsolver, smem);
}
}  // namespace jx
