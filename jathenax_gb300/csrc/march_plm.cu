// Register-marching stage kernels for the plm reconstruction: dispatch by
// Riemann solver to the march_plm_<solver>.cu translation units, which
// hold the instantiations (one per solver, so the build compiles them in
// parallel).
#include "jx_internal.h"

namespace jx {
cudaError_t launch_march_plm_llf(int dtype, const StageParams& p, dim3 grid, cudaStream_t s);
cudaError_t launch_batch_march_plm_llf(int dtype, int nv, int nc, int ring, int form, const StageParams* params, const int* offsets,
                                  int nsolves, int nwork, dim3 grid, cudaStream_t s);
int march_blocks_per_sm_plm_llf(int dtype, int nv, int nc, int kind);
cudaError_t launch_march_plm_hlle(int dtype, const StageParams& p, dim3 grid, cudaStream_t s);
cudaError_t launch_batch_march_plm_hlle(int dtype, int nv, int nc, int ring, int form, const StageParams* params, const int* offsets,
                                  int nsolves, int nwork, dim3 grid, cudaStream_t s);
int march_blocks_per_sm_plm_hlle(int dtype, int nv, int nc, int kind);
cudaError_t launch_march_plm_roe(int dtype, const StageParams& p, dim3 grid, cudaStream_t s);
cudaError_t launch_batch_march_plm_roe(int dtype, int nv, int nc, int ring, int form, const StageParams* params, const int* offsets,
                                  int nsolves, int nwork, dim3 grid, cudaStream_t s);
int march_blocks_per_sm_plm_roe(int dtype, int nv, int nc, int kind);

cudaError_t launch_march_plm(int dtype, int rsolver, const StageParams& p, dim3 grid, cudaStream_t s) {
  switch (rsolver) {
    case JX_LLF: return launch_march_plm_llf(dtype, p, grid, s);
    case JX_HLLE: return launch_march_plm_hlle(dtype, p, grid, s);
    case JX_ROE: return launch_march_plm_roe(dtype, p, grid, s);
  }
  return cudaErrorInvalidValue;
}
cudaError_t launch_batch_march_plm(int dtype, int rsolver, int nv, int nc, int ring, int form, const StageParams* params, const int* offsets,
                                  int nsolves, int nwork, dim3 grid, cudaStream_t s) {
  switch (rsolver) {
    case JX_LLF: return launch_batch_march_plm_llf(dtype, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
    case JX_HLLE: return launch_batch_march_plm_hlle(dtype, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
    case JX_ROE: return launch_batch_march_plm_roe(dtype, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
  }
  return cudaErrorInvalidValue;
}
int march_blocks_per_sm_plm(int dtype, int rsolver, int nv, int nc, int kind) {
  switch (rsolver) {
    case JX_LLF: return march_blocks_per_sm_plm_llf(dtype, nv, nc, kind);
    case JX_HLLE: return march_blocks_per_sm_plm_hlle(dtype, nv, nc, kind);
    default: return march_blocks_per_sm_plm_roe(dtype, nv, nc, kind);
  }
}
}  // namespace jx
