// cp.async row ring shared by the float32 marching kernels: each lane
// stages its own cells of upcoming rows in shared memory.
#pragma once
#include "jx_internal.h"
#include "jx_stage_fast.cuh"

namespace jx {

// Row ring of the float32 single-solve walk on tall tiles: rows of U arrive
// by cp.async three rows ahead of their use and rows of V three rows ahead
// of the RK combine, into shared memory that only the copying lane reads
// (slot [row][column h][lane], 16 bytes a cell, so a warp's accesses are
// conflict-free). kRingU rows of U stay until the combine of the row has
// read them too (its U then comes from the ring, not from L1/L2); kRingV
// rows of V. No register holds a row in flight. Measured on GB300 at 4096²
// (ppm4+roe, float32, RK3 stage 2): 0.2957 -> 0.2814 ms on 58 x 121 tiles,
// 0.3144 -> 0.2792 ms on 90 x 106; on the 8-row tiles of a 1024² grid it
// was 7 % slower (0.027 -> 0.029 ms), so tiles shorter than kRingMinRows
// keep the register path. The bits are the same either way.
constexpr int kRingU = 8, kRingV = 4, kRingAhead = 3;
// Where the ring is built (march_ring_built): float32, not DC (nearest to
// the HBM bound, 0.175 ms per 4096² stage on the register path against 0.193
// with the ring) and not WENO-Z with two or three columns per lane (58 x 121:
// 1.478 against 1.506 ms); PLM, PPM4, PPMX and one-column WENO-Z gain 1-22 %.
template <typename R, int RECON, int NC> constexpr bool march_ring_on() {
  return march_ring_built(sizeof(R) == 4, RECON, NC);
}
template <int NC> __host__ __device__ constexpr int march_ring_bytes() { return (kRingU + kRingV) * NC * 32 * 16; }

__device__ __forceinline__ void cp_async_16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_4(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One cell (NV floats) from global to its ring slot.
template <int NV>
__device__ __forceinline__ void ring_copy(float4* slot, const float* g) {
  if constexpr (NV == 4) {
    cp_async_16(slot, g);
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) cp_async_4(reinterpret_cast<float*>(slot) + v, g + v);
  }
}

template <int NV>
__device__ __forceinline__ Cell4<float> ring_read(const float4* slot) {
  const float4 t = *slot;
  Cell4<float> c;
  c.v[0] = t.x;
  c.v[1] = t.y;
  c.v[2] = t.z;
  c.v[3] = NV == 4 ? t.w : 0.0f;
  return c;
}

}  // namespace jx
