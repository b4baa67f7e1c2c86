// Fast path of the fused RK-stage kernel for 3 or 4 variables (the reference's
// hydro state, optionally with one tracer), with the tile width fixed at 32.
//
// Same phases and arithmetic as stage_kernel (jx_stage.cuh), organised for a
// lower instruction count per cell:
//   * compile-time variable count and tile width: every thread->work index
//     split divides by a constant and every per-variable loop unrolls;
//   * cell-major shared memory: the (up to) four values of a cell sit in one
//     16-byte (float) or 32-byte (double) vector, so a stencil point costs one
//     or two 128-bit shared loads instead of four 32/64-bit ones;
//   * every tile computes a full 32 x TY block (ragged right/bottom tiles read
//     periodically wrapped neighbours) and masks only the final writes, so no
//     loop bound depends on the tile;
//   * with 4 variables the state is read and written with 128-bit global
//     accesses (the host only selects this kernel for 16-byte aligned arrays).
#pragma once
#include "jx_device.cuh"
#include "jx_internal.h"

namespace jx {

constexpr int kFastTX = 32;

template <typename R> struct alignas(16) Cell4 {
  R v[4];
};

template <typename R, int NV>
__device__ __forceinline__ Cell4<R> load_cell(const R* __restrict__ p) {
  Cell4<R> c;
  if constexpr (NV == 4 && sizeof(R) == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    c.v[0] = t.x; c.v[1] = t.y; c.v[2] = t.z; c.v[3] = t.w;
  } else if constexpr (NV == 4 && sizeof(R) == 8) {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    c.v[0] = a.x; c.v[1] = a.y; c.v[2] = b.x; c.v[3] = b.y;
  } else {
#pragma unroll
    for (int k = 0; k < NV; ++k) c.v[k] = p[k];
#pragma unroll
    for (int k = NV; k < 4; ++k) c.v[k] = R(0);
  }
  return c;
}

template <typename R, int NV>
__device__ __forceinline__ void store_cell(R* __restrict__ p, const Cell4<R>& c) {
  if constexpr (NV == 4 && sizeof(R) == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(c.v[0], c.v[1], c.v[2], c.v[3]);
  } else if constexpr (NV == 4 && sizeof(R) == 8) {
    reinterpret_cast<double2*>(p)[0] = make_double2(c.v[0], c.v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(c.v[2], c.v[3]);
  } else {
#pragma unroll
    for (int k = 0; k < NV; ++k) p[k] = c.v[k];
  }
}

// Scalar stores for the optional trace outputs (any alignment).
template <typename R, int NV>
__device__ __forceinline__ void store_cell_scalar(void* base, size_t cell, const Cell4<R>& c) {
  if (!base) return;
  R* p = static_cast<R*>(base) + cell * NV;
#pragma unroll
  for (int k = 0; k < NV; ++k) p[k] = c.v[k];
}

__device__ __forceinline__ int wrap_fast(int i, int n) {
  return (unsigned)i < (unsigned)n ? i : wrap_index(i, n);
}

template <typename R> struct FastTile {
  Cell4<R> *W, *Fx, *Fy, *A, *Rt;
  int TY;
};

// Cells per shared plane of the fast kernel.
__host__ __device__ inline void fast_planes(int recon, int ty, int* w, int* fx, int* fy, int* a, int* r) {
  const int h = recon == JX_DC ? 1 : (recon == JX_PLM ? 2 : 3);
  const int tx = kFastTX;
  *w = (tx + 2 * h) * (ty + 2 * h);
  *fx = ty * (tx + 1);
  *fy = (ty + 1) * tx;
  const int ax = ty * (tx + 3), ay = (ty + 3) * tx;
  *a = (recon == JX_PPM4 || recon == JX_PPMX) ? (ax > ay ? ax : ay) : 0;
  *r = *fx > *fy ? *fx : *fy;
}

template <int DIR, typename R, int RECON, int RS, int NV>
__device__ __forceinline__ void fast_sweep(const StageParams& p, const StageConsts<R>& k, FastTile<R>& t, int x0,
                                           int y0) {
  using Tr = ReconTraits<RECON>;
  using N = Num<R>;
  constexpr int H = Tr::kHalo;
  constexpr int TX = kFastTX;
  constexpr int PW = TX + 2 * H;
  constexpr bool kFaceFloor = RECON == 3 || RECON == 4;  // fluxes.py:128-130
  constexpr int ST = DIR == 0 ? 1 : PW;                  // stencil stride in W
  const int TY = t.TY;
  const int tid = threadIdx.x;
  Cell4<R>* F = DIR == 0 ? t.Fx : t.Fy;
  // Work item -> (line, position q along the line); lines are rows for the x
  // sweep and columns for the y sweep; consecutive threads move along x.
  auto split = [&](int idx, int len, int& ln, int& q) {
    if (DIR == 0) { ln = idx / len; q = idx - ln * len; }  // len is a constant
    else { ln = idx % TX; q = idx / TX; }
  };
  auto wcell = [&](int ln, int q) { return DIR == 0 ? (ln + H) * PW + (q + H) : (q + H) * PW + (ln + H); };
  auto fidx = [&](int ln, int q) { return DIR == 0 ? ln * (TX + 1) + q : q * TX + ln; };
  auto aidx = [&](int ln, int q) { return DIR == 0 ? ln * (TX + 3) + q + 1 : (q + 1) * TX + ln; };
  const int nlines = DIR == 0 ? TY : TX;
  const int n = DIR == 0 ? TX : TY;  // cells per line

  if constexpr (Tr::kFaceShared) {
    const int len = n + 3;  // faces -1 .. n+1
    const int total = DIR == 0 ? TY * (TX + 3) : (TY + 3) * TX;
    for (int idx = tid; idx < total; idx += kStageThreads) {
      int ln, q;
      split(idx, DIR == 0 ? TX + 3 : len, ln, q);
      q -= 1;
      const int s = wcell(ln, q);
      const Cell4<R> w0 = t.W[s - 2 * ST], w1 = t.W[s - ST], w2 = t.W[s], w3 = t.W[s + ST];
      Cell4<R> a;
#pragma unroll
      for (int v = 0; v < NV; ++v) a.v[v] = face_value<RECON>(w0.v[v], w1.v[v], w2.v[v], w3.v[v]);
#pragma unroll
      for (int v = NV; v < 4; ++v) a.v[v] = R(0);
      t.A[aidx(ln, q)] = a;
    }
    __syncthreads();
  }

  {
    const int total = DIR == 0 ? TY * (TX + 2) : (TY + 2) * TX;  // cells -1 .. n
    for (int idx = tid; idx < total; idx += kStageThreads) {
      int ln, q;
      split(idx, TX + 2, ln, q);
      q -= 1;
      const int s = wcell(ln, q);
      const Cell4<R> c = t.W[s];
      Cell4<R> m1 = c, p1 = c, m2 = c, p2 = c;
      if constexpr (H >= 2 && RECON != 2) {  // ppm4's limiter needs only the cell and its faces
        m1 = t.W[s - ST];
        p1 = t.W[s + ST];
      }
      if constexpr (H >= 3 && RECON != 2) {
        m2 = t.W[s - 2 * ST];
        p2 = t.W[s + 2 * ST];
      }
      Cell4<R> lf = c, hf = c;
      if constexpr (Tr::kFaceShared) {
        lf = t.A[aidx(ln, q)];
        hf = t.A[aidx(ln, q + 1)];
      }
      Cell4<R> lo, hi;
#pragma unroll
      for (int v = 0; v < NV; ++v)
        cell_edges<RECON>(m2.v[v], m1.v[v], c.v[v], p1.v[v], p2.v[v], lf.v[v], hf.v[v], lo.v[v], hi.v[v]);
#pragma unroll
      for (int v = NV; v < 4; ++v) lo.v[v] = hi.v[v] = R(0);
      if constexpr (kFaceFloor) {
        lo.v[0] = N::max(lo.v[0], k.dfloor);
        hi.v[0] = N::max(hi.v[0], k.dfloor);
      }
      if (q + 1 <= n) F[fidx(ln, q + 1)] = hi;  // left state of face q+1
      if (q >= 0) t.Rt[fidx(ln, q)] = lo;       // right state of face q
    }
    __syncthreads();
  }

  {
    Gas<R> gas;
    gas.cs = k.cs;
    gas.cs2 = k.cs2;
    gas.inv_cs = k.inv_cs;
    gas.half_inv_cs = k.half_inv_cs;
    gas.quarter_inv_cs = R(0.5) * k.half_inv_cs;
    const R* __restrict__ tau = static_cast<const R*>(p.tau);
    constexpr int nn = DIR == 0 ? 1 : 2, tt = DIR == 0 ? 2 : 1;
    const int total = DIR == 0 ? TY * (TX + 1) : (TY + 1) * TX;  // faces 0 .. n
    for (int idx = tid; idx < total; idx += kStageThreads) {
      int ln, q;
      split(idx, TX + 1, ln, q);
      const int fo = fidx(ln, q);
      const Cell4<R> L = F[fo], Rv = t.Rt[fo];
      R f0, fn, ft;
      riemann<RS>(L.v[0], Rv.v[0], L.v[nn], Rv.v[nn], L.v[tt], Rv.v[tt], gas, f0, fn, ft);
      Cell4<R> f;
      f.v[0] = f0;
      f.v[1] = DIR == 0 ? fn : ft;
      f.v[2] = DIR == 0 ? ft : fn;
      f.v[3] = R(0);
      const int r = DIR == 0 ? ln : q, c = DIR == 0 ? q : ln;  // tile cell on the high side
      if (p.visc_on) {
        const int sb = (r + H) * PW + (c + H);
        const int sa = sb - ST;
        const Cell4<R> b = t.W[sb], a = t.W[sa];
        // Transverse neighbours one cell beyond the face on either side.
        constexpr int TS = DIR == 0 ? PW : 1;
        const Cell4<R> bp = t.W[sb + TS], ap = t.W[sa + TS], bm = t.W[sb - TS], am = t.W[sa - TS];
        viscous_face<DIR, R>(p.smag_on, k.nu, k.smag_c, DIR == 0 ? k.inv_dx : k.inv_dy,
                             DIR == 0 ? k.inv_4dy : k.inv_4dx, a.v[0], b.v[0], a.v[1], a.v[2], b.v[1], b.v[2],
                             bp.v[1] + ap.v[1], bp.v[2] + ap.v[2], bm.v[1] + am.v[1], bm.v[2] + am.v[2], f.v[1],
                             f.v[2]);
      }
      if (tau != nullptr) {
        const int gy = wrap_fast(y0 + r, p.ny), gx = wrap_fast(x0 + c, p.nx);
        const int ay = DIR == 0 ? gy : wrap_fast(y0 + r - 1, p.ny);
        const int ax = DIR == 0 ? wrap_fast(x0 + c - 1, p.nx) : gx;
        const R* tb = tau + ((size_t)gy * p.nx + gx) * 3;
        const R* ta = tau + ((size_t)ay * p.nx + ax) * 3;
        constexpr int k0 = DIR == 0 ? 0 : 1;
        f.v[1] = add_half_sum(f.v[1], ta[k0], tb[k0]);
        f.v[2] = add_half_sum(f.v[2], ta[k0 + 1], tb[k0 + 1]);
      }
#pragma unroll
      for (int v = 3; v < NV; ++v) f.v[v] = scalar_flux(f0, L.v[v], Rv.v[v]);
      if (p.trace_on && q < n && y0 + r < p.ny && x0 + c < p.nx) {
        const size_t cell = (size_t)(y0 + r) * p.nx + (x0 + c);
        store_cell_scalar<R, NV>(DIR == 0 ? p.trace.left_x : p.trace.left_y, cell, L);
        store_cell_scalar<R, NV>(DIR == 0 ? p.trace.right_x : p.trace.right_y, cell, Rv);
        store_cell_scalar<R, NV>(DIR == 0 ? p.trace.flux_x : p.trace.flux_y, cell, f);
      }
      F[fo] = f;
    }
    __syncthreads();
  }
  (void)nlines;
}

// One 32 x TY tile of one solve. `tile` indexes the solve's tiles (row-major);
// its CFL partial goes to slot `tile` of the solve's workspace, so results do
// not depend on which block or launch processes the tile.
template <typename R, int RECON, int RS, int NV>
__device__ __forceinline__ void fast_tile(const StageParams& p, int tile, int ntiles, unsigned char* smem_raw,
                                          double* red, R* s_sdt) {
  using N = Num<R>;
  constexpr int H = ReconTraits<RECON>::kHalo;
  constexpr int TX = kFastTX;
  constexpr int PW = TX + 2 * H;
  const StageConsts<R>& k = stage_consts<R>(p);

  const int tid = threadIdx.x;
  const int TY = p.ty;
  const int bx = tile % p.tiles_x, by = tile / p.tiles_x;
  const int x0 = bx * TX, y0 = by * TY;
  int pw, pfx, pfy, pa, pr;
  fast_planes(RECON, TY, &pw, &pfx, &pfy, &pa, &pr);
  FastTile<R> t;
  t.TY = TY;
  t.W = reinterpret_cast<Cell4<R>*>(smem_raw);
  t.Fx = t.W + pw;
  t.Fy = t.Fx + pfx;
  t.A = t.Fy + pfy;
  t.Rt = t.A + pa;

  const R* __restrict__ U = static_cast<const R*>(p.U);
  if (tid == 0) *s_sdt = static_cast<R>(p.beta * p.clock->dt);

  const int PH = TY + 2 * H;
  for (int idx = tid; idx < PW * PH; idx += kStageThreads) {
    const int ly = idx / PW, lx = idx - ly * PW;
    const int gy = wrap_fast(y0 + ly - H, p.ny), gx = wrap_fast(x0 + lx - H, p.nx);
    const Cell4<R> u = load_cell<R, NV>(U + ((size_t)gy * p.nx + gx) * NV);
    Cell4<R> w;
    const R rho = N::lt(u.v[0], k.dfloor) ? k.dfloor : u.v[0];
    const R inv = Num<R>::rcp(rho);
    w.v[0] = rho;
#pragma unroll
    for (int v = 1; v < 4; ++v) w.v[v] = v < NV ? Ops<R>::mul(inv, u.v[v]) : R(0);
    t.W[idx] = w;
  }
  __syncthreads();

  fast_sweep<0, R, RECON, RS, NV>(p, k, t, x0, y0);
  fast_sweep<1, R, RECON, RS, NV>(p, k, t, x0, y0);

  const R* __restrict__ V = static_cast<const R*>(p.V);
  R* Uo = static_cast<R*>(p.Uout);
  R* Vo = static_cast<R*>(p.Vout);
  const R sdt = *s_sdt;
  const R kdrag = sdt * k.drag;
  const R ncx = -(sdt * k.inv_dx), ncy = -(sdt * k.inv_dy);
  R vmax0 = R(0), vmax1 = R(0);
  // The combine loop is instantiated per (blend form, RK4 delta, drag, CFL
  // partials) so that no float64 work of an unused form is evaluated and
  // then discarded.
  auto combine = [&](auto blend_tag, auto delta_tag, auto drag_tag, auto cfl_tag) {
    constexpr bool kBlend = decltype(blend_tag)::value;
    constexpr bool kDelta = decltype(delta_tag)::value;
    constexpr bool kDrag = decltype(drag_tag)::value;
    constexpr bool kCfl = decltype(cfl_tag)::value;
    for (int idx = tid; idx < TY * TX; idx += kStageThreads) {
      const int r = idx / TX, c = idx - r * TX;
      if (y0 + r >= p.ny || x0 + c >= p.nx) continue;
      const size_t cell = (size_t)(y0 + r) * p.nx + (x0 + c);
      const Cell4<R> w = t.W[(r + H) * PW + (c + H)];
      const Cell4<R> fxl = t.Fx[r * (TX + 1) + c], fxr = t.Fx[r * (TX + 1) + c + 1];
      const Cell4<R> fyl = t.Fy[r * TX + c], fyr = t.Fy[(r + 1) * TX + c];
      Cell4<R> u = load_cell<R, NV>(U + cell * NV);
      u.v[0] = w.v[0];  // the floored density
      Cell4<R> vs = load_cell<R, NV>(V + cell * NV);
      if (p.floor_v) vs.v[0] = N::lt(vs.v[0], k.dfloor) ? k.dfloor : vs.v[0];
      Cell4<R> un;
  #pragma unroll
      for (int v = 0; v < NV; ++v) {
        if (kDelta) vs.v[v] = delta_update(vs.v[v], k.delta, u.v[v]);
        un.v[v] = rk_combine<R>(kBlend, k.g0, k.g1, u.v[v], vs.v[v], fxr.v[v] - fxl.v[v], fyr.v[v] - fyl.v[v], ncx,
                                ncy);
      }
      un.v[3] = NV == 4 ? un.v[3] : R(0);
      if (kDrag) {
        un.v[1] = drag_term(un.v[1], kdrag * w.v[0], w.v[1]);
        un.v[2] = drag_term(un.v[2], kdrag * w.v[0], w.v[2]);
      }
      if (p.trace_on) {
        store_cell_scalar<R, NV>(p.trace.saved, cell, vs);
        store_cell_scalar<R, NV>(p.trace.conserved, cell, un);
        store_cell_scalar<R, NV>(p.trace.primitives, cell, w);
      }
      if (kDelta && Vo) store_cell<R, NV>(Vo + cell * NV, vs);
      if (p.floor_out) un.v[0] = N::lt(un.v[0], k.dfloor) ? k.dfloor : un.v[0];
      store_cell<R, NV>(Uo + cell * NV, un);
      if (kCfl) {
        const R inv = Num<R>::rcp(un.v[0]);
        vmax0 = N::nanmax_pos(vmax0, signal_speed(inv, un.v[1], k.cs));
        vmax1 = N::nanmax_pos(vmax1, signal_speed(inv, un.v[2], k.cs));
      }
    }
  };
  auto with_cfl = [&](auto b, auto d, auto g) {
    if (p.want_cfl) combine(b, d, g, Flag<true>{});
    else combine(b, d, g, Flag<false>{});
  };
  auto with_drag = [&](auto b, auto d) {
    if (p.drag_on) with_cfl(b, d, Flag<true>{});
    else with_cfl(b, d, Flag<false>{});
  };
  auto with_delta = [&](auto b) {
    if (p.has_delta) with_drag(b, Flag<true>{});
    else with_drag(b, Flag<false>{});
  };
  if (p.blend) with_delta(Flag<true>{});
  else with_delta(Flag<false>{});
  if (p.want_cfl) {
    double vmax[2] = {static_cast<double>(vmax0), static_cast<double>(vmax1)};
    block_nan_max<2>(vmax, red);
    if (tid == 0) {
      p.partials[(size_t)tile * kCflSlots + 0] = vmax[0];
      p.partials[(size_t)tile * kCflSlots + 1] = vmax[1];
      p.partials[(size_t)tile * kCflSlots + 2] = 0.0;
      if (tile == 0) p.header->n_cfl = ntiles;
    }
  }
}

template <typename R, int RECON, int RS, int NV>
__global__ void __launch_bounds__(kStageThreads) stage_kernel_fast(const StageParams p) {
  if (p.clock->done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32 * 2];
  __shared__ R s_sdt;
  fast_tile<R, RECON, RS, NV>(p, blockIdx.x, gridDim.x, smem_raw, red, &s_sdt);
}

// Persistent stage kernel over many solves (one group: same precision,
// reconstruction and Riemann solver; 3 or 4 variables per solve). Work item w
// is tile w - tile_offset[i] of solve i. Blocks take work items round-robin;
// a solve that is done, or whose integrator has fewer stages, is skipped.
template <typename R, int RECON, int RS>
__global__ void __launch_bounds__(kStageThreads) stage_kernel_batch(const StageParams* __restrict__ params,
                                                                    const int* __restrict__ tile_offset,
                                                                    int nsolves, int nwork) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32 * 2];
  __shared__ R s_sdt;
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    int lo = 0, hi = nsolves - 1;  // last solve whose offset <= w
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tile_offset[mid] <= w) lo = mid;
      else hi = mid - 1;
    }
    const StageParams& p = params[lo];
    if (p.skip || p.clock->done) continue;
    const int tile = w - tile_offset[lo];
    const int ntiles = tile_offset[lo + 1] - tile_offset[lo];
    __syncthreads();  // the previous tile's last readers of shared memory are done
    if (p.nv == 3) fast_tile<R, RECON, RS, 3>(p, tile, ntiles, smem_raw, red, &s_sdt);
    else fast_tile<R, RECON, RS, 4>(p, tile, ntiles, smem_raw, red, &s_sdt);
  }
}

template <typename R, int RECON, int RS, int NV>
cudaError_t launch_fast_one(const StageParams& p, dim3 grid, size_t smem, cudaStream_t s) {
  auto kernel = stage_kernel_fast<R, RECON, RS, NV>;
  static int granted[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if ((int)smem > granted[dev]) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    granted[dev] = (int)smem;
  }
  kernel<<<grid, kStageThreads, smem, s>>>(p);
  return cudaGetLastError();
}

template <typename R, int RECON, int NV>
cudaError_t launch_fast_rs(int rsolver, const StageParams& p, dim3 grid, size_t smem, cudaStream_t s) {
  switch (rsolver) {
    case JX_LLF: return launch_fast_one<R, RECON, JX_LLF, NV>(p, grid, smem, s);
    case JX_HLLE: return launch_fast_one<R, RECON, JX_HLLE, NV>(p, grid, smem, s);
    case JX_ROE: return launch_fast_one<R, RECON, JX_ROE, NV>(p, grid, smem, s);
  }
  return cudaErrorInvalidValue;
}

template <typename R, int RECON>
cudaError_t launch_batch_rs(int rsolver, const StageParams* params, const int* offsets, int nsolves, int nwork,
                            dim3 grid, size_t smem, cudaStream_t s) {
  auto pick = [&](auto kernel) -> cudaError_t {
    static int granted[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if ((int)smem > granted[dev]) {
      cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      granted[dev] = (int)smem;
    }
    kernel<<<grid, kStageThreads, smem, s>>>(params, offsets, nsolves, nwork);
    return cudaGetLastError();
  };
  switch (rsolver) {
    case JX_LLF: return pick(stage_kernel_batch<R, RECON, JX_LLF>);
    case JX_HLLE: return pick(stage_kernel_batch<R, RECON, JX_HLLE>);
    case JX_ROE: return pick(stage_kernel_batch<R, RECON, JX_ROE>);
  }
  return cudaErrorInvalidValue;
}

template <int RECON>
cudaError_t launch_batch_recon(int dtype, int rsolver, const StageParams* params, const int* offsets, int nsolves,
                               int nwork, dim3 grid, size_t smem, cudaStream_t s) {
  if (dtype == JX_F64) return launch_batch_rs<double, RECON>(rsolver, params, offsets, nsolves, nwork, grid, smem, s);
  return launch_batch_rs<float, RECON>(rsolver, params, offsets, nsolves, nwork, grid, smem, s);
}

// Blocks of the persistent batch kernel that fit on one SM.
template <typename R, int RECON, int RS>
int batch_blocks_per_sm_rs(size_t smem) {
  int n = 0;
  cudaFuncSetAttribute(stage_kernel_batch<R, RECON, RS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage_kernel_batch<R, RECON, RS>, kStageThreads, smem);
  return n;
}

template <int RECON>
int batch_blocks_per_sm_recon(int dtype, int rsolver, size_t smem) {
  if (dtype == JX_F64) {
    if (rsolver == JX_LLF) return batch_blocks_per_sm_rs<double, RECON, JX_LLF>(smem);
    if (rsolver == JX_HLLE) return batch_blocks_per_sm_rs<double, RECON, JX_HLLE>(smem);
    return batch_blocks_per_sm_rs<double, RECON, JX_ROE>(smem);
  }
  if (rsolver == JX_LLF) return batch_blocks_per_sm_rs<float, RECON, JX_LLF>(smem);
  if (rsolver == JX_HLLE) return batch_blocks_per_sm_rs<float, RECON, JX_HLLE>(smem);
  return batch_blocks_per_sm_rs<float, RECON, JX_ROE>(smem);
}

template <int RECON>
cudaError_t launch_fast_recon(int dtype, int rsolver, const StageParams& p, dim3 grid, size_t smem,
                              cudaStream_t s) {
  if (dtype == JX_F64) {
    return p.nv == 3 ? launch_fast_rs<double, RECON, 3>(rsolver, p, grid, smem, s)
                     : launch_fast_rs<double, RECON, 4>(rsolver, p, grid, smem, s);
  }
  return p.nv == 3 ? launch_fast_rs<float, RECON, 3>(rsolver, p, grid, smem, s)
                   : launch_fast_rs<float, RECON, 4>(rsolver, p, grid, smem, s);
}

}  // namespace jx
