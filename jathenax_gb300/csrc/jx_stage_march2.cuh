// Float32 marching stage kernel that walks two tiles at once as float32
// pairs (PPM4 reconstruction, Roe solver, 3 or 4 variables, the lean
// inviscid forms).
//
// The single-tile marching kernel (jx_stage_march.cuh) is bound by
// instruction issue. Here one warp takes tile A and tile B (58 x TY each, two
// columns per lane as there), and every value the walk holds is a float2
// pair (tile A's, tile B's) of the same cell position: the primitives'
// window, face values, edges, fluxes. Every add, multiply and FMA of the
// y and x sweeps is one packed Blackwell instruction (__fadd2_rn,
// __fmul2_rn, __ffma2_rn) for both tiles; comparisons, selects, min/max,
// the SFU reciprocal and root and the warp shuffles stay per half. The pairs
// never mix cells of one tile, so no value has to be moved between register
// pairs: a neighbour lane's pair arrives by two shuffles, a neighbour column
// of the same lane is the lane's other pair. Primitive recovery and the RK
// combine work per cell (their operands come from 16-byte loads).
//
// Each packed operation rounds each half exactly as the corresponding
// explicitly rounded float32 operation of jx_device.cuh (a - b is formed as
// fma(b, -1, a), which rounds once, as a - b does), so the results are the
// same bits as every other float32 stage kernel's (tested).
#pragma once
#include "jx_device.cuh"
#include "jx_internal.h"
#include "jx_stage_fast.cuh"

namespace jx {
namespace pk {

using F2 = float2;

__device__ __forceinline__ F2 splat(float a) { return make_float2(a, a); }
__device__ __forceinline__ F2 add(F2 a, F2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ F2 mul(F2 a, F2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ F2 fma(F2 a, F2 b, F2 c) { return __ffma2_rn(a, b, c); }
// a - b rounded once: fma(b, -1, a) (the product is exact).
__device__ __forceinline__ F2 sub(F2 a, F2 b) { return __ffma2_rn(b, splat(-1.f), a); }
__device__ __forceinline__ F2 neg(F2 a) { return __fmul2_rn(a, splat(-1.f)); }
__device__ __forceinline__ F2 abs2(F2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ F2 min2(F2 a, F2 b) { return make_float2(fminf(a.x, b.x), fminf(a.y, b.y)); }
__device__ __forceinline__ F2 max2(F2 a, F2 b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
__device__ __forceinline__ F2 rcp2(F2 a) { return make_float2(Num<float>::rcp(a.x), Num<float>::rcp(a.y)); }
__device__ __forceinline__ F2 root2(F2 a) { return make_float2(Num<float>::root(a.x), Num<float>::root(a.y)); }
__device__ __forceinline__ F2 sel(bool cx, bool cy, F2 a, F2 b) { return make_float2(cx ? a.x : b.x, cy ? a.y : b.y); }

struct PCell {
  F2 v[4];
};

template <int NV>
__device__ __forceinline__ PCell shfl_up(const PCell& c, int d) {
  PCell o;
#pragma unroll
  for (int v = 0; v < 4; ++v)
    o.v[v] = v < NV ? make_float2(__shfl_up_sync(0xffffffffu, c.v[v].x, d), __shfl_up_sync(0xffffffffu, c.v[v].y, d))
                    : splat(0.f);
  return o;
}

template <int NV>
__device__ __forceinline__ PCell shfl_down(const PCell& c, int d) {
  PCell o;
#pragma unroll
  for (int v = 0; v < 4; ++v)
    o.v[v] = v < NV ? make_float2(__shfl_down_sync(0xffffffffu, c.v[v].x, d),
                                  __shfl_down_sync(0xffffffffu, c.v[v].y, d))
                    : splat(0.f);
  return o;
}

// ppm4_face (float32): the fourth-order interpolant bounded by the two
// neighbours; min/max per half in the scalar operand order.
__device__ __forceinline__ F2 ppm4_face2(F2 w0, F2 w1, F2 w2, F2 w3) {
  const F2 e = mul(fma(splat(7.f), add(w2, w1), neg(add(w0, w3))), splat(float(1.0 / 12.0)));
  return min2(max2(e, min2(w2, w1)), max2(w2, w1));
}

// ppm4_cell (float32 branch).
__device__ __forceinline__ void ppm4_cell2(F2 c, F2 lo_face, F2 hi_face, F2& lo, F2& hi) {
  const F2 dh = sub(hi_face, c), dl = sub(lo_face, c);
  const F2 p = mul(dh, dl);
  const F2 dh2 = mul(splat(2.f), abs2(dh)), dl2 = mul(splat(2.f), abs2(dl));
  const bool flat_x = p.x >= 0.f, flat_y = p.y >= 0.f;
  const bool slo_x = fabsf(dl.x) >= dh2.x, slo_y = fabsf(dl.y) >= dh2.y;
  const bool shi_x = fabsf(dh.x) >= dl2.x, shi_y = fabsf(dh.y) >= dl2.y;
  const F2 l2 = sel(slo_x, slo_y, fma(splat(-2.f), dh, c), lo_face);
  const F2 h2 = sel(shi_x, shi_y, fma(splat(-2.f), dl, c), hi_face);
  lo = sel(flat_x, flat_y, c, l2);
  hi = sel(flat_x, flat_y, c, h2);
}

// flux_roe_f32, both halves at once (fluxes.py:134-172).
__device__ __forceinline__ void roe2(F2 dl, F2 dr, F2 ul, F2 ur, F2 tl, F2 tr, const Gas<float>& g, F2& f0, F2& f1,
                                     F2& f2) {
  const F2 cs = splat(g.cs), cs2 = splat(g.cs2), half = splat(0.5f), hic = splat(g.half_inv_cs);
  const F2 ml = mul(dl, ul), mr = mul(dr, ur);
  const F2 ql = mul(dl, tl), qr = mul(dr, tr);
  const F2 s0 = add(ml, mr);
  const F2 s1 = fma(ml, ul, fma(mr, ur, mul(cs2, add(dl, dr))));
  const F2 s2 = fma(ml, tl, mul(mr, tr));
  const F2 r = mul(root2(dl), root2(dr));
  const F2 inv = rcp2(add(dl, r));
  const F2 u = mul(fma(r, ur, ml), inv);
  const F2 t = mul(fma(r, tr, ql), inv);
  const F2 lm = sub(u, cs), lp = add(u, cs);
  const F2 jd = sub(dr, dl), jm = sub(mr, ml), jq = sub(qr, ql);
  const F2 hu = mul(u, hic);
  const F2 jmc = mul(jm, hic);
  const F2 am = fma(jd, add(half, hu), neg(jmc));
  const F2 ap = fma(jd, sub(half, hu), jmc);
  const F2 az = fma(jd, neg(t), jq);
  const F2 wm = mul(abs2(lm), am), wz = mul(abs2(u), az), wp = mul(abs2(lp), ap);
  const F2 wmp = add(wm, wp);
  const F2 dstar = add(dl, am);
  const F2 dstar2 = add(dstar, ap);
  f0 = mul(half, sub(s0, wmp));
  f1 = mul(half, sub(s1, fma(wm, lm, mul(wp, lp))));
  f2 = mul(half, sub(s2, fma(wmp, t, wz)));
  const bool bad_x = dstar.x < 0.f || dstar2.x < 0.f, bad_y = dstar.y < 0.f || dstar2.y < 0.f;
  if (__builtin_expect(bad_x || bad_y, 0)) {  // positivity fix: rare
    const F2 sp = mul(half, max2(add(abs2(ul), cs), add(abs2(ur), cs)));
    const F2 nsp = neg(sp);
    f0 = sel(bad_x, bad_y, fma(nsp, jd, mul(half, s0)), f0);
    f1 = sel(bad_x, bad_y, fma(nsp, jm, mul(half, s1)), f1);
    f2 = sel(bad_x, bad_y, fma(nsp, jq, mul(half, s2)), f2);
  }
}

// face_flux_cells<roe> for both halves: Riemann flux in x/y component order
// plus passive-scalar upwinding.
template <int DIR, int NV>
__device__ __forceinline__ PCell face_flux2(const PCell& L, const PCell& Rv, const Gas<float>& g) {
  constexpr int nn = DIR == 0 ? 1 : 2, tt = DIR == 0 ? 2 : 1;
  F2 f0, fn, ft;
  roe2(L.v[0], Rv.v[0], L.v[nn], Rv.v[nn], L.v[tt], Rv.v[tt], g, f0, fn, ft);
  PCell f;
  f.v[0] = f0;
  f.v[1] = DIR == 0 ? fn : ft;
  f.v[2] = DIR == 0 ? ft : fn;
  f.v[3] = splat(0.f);
#pragma unroll
  for (int v = 3; v < NV; ++v)
    f.v[v] = mul(f0, sel(f0.x >= 0.f, f0.y >= 0.f, L.v[v], Rv.v[v]));
  return f;
}

template <int NV>
__device__ __forceinline__ PCell faces2(const PCell& w0, const PCell& w1, const PCell& w2, const PCell& w3) {
  PCell a;
#pragma unroll
  for (int v = 0; v < 4; ++v) a.v[v] = v < NV ? ppm4_face2(w0.v[v], w1.v[v], w2.v[v], w3.v[v]) : splat(0.f);
  return a;
}

template <int NV>
__device__ __forceinline__ void edges2(const PCell& c, const PCell& lf, const PCell& hf, PCell& lo, PCell& hi) {
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    if (v < NV) ppm4_cell2(c.v[v], lf.v[v], hf.v[v], lo.v[v], hi.v[v]);
    else lo.v[v] = hi.v[v] = splat(0.f);
  }
}

// The pair of recovered cells (tile A's cell a, tile B's cell b): the
// density floor, then the primitives, per cell as recover_cell does.
template <int NV>
__device__ __forceinline__ PCell recover2(const Cell4<float>& a, const Cell4<float>& b, float dfloor) {
  const float ra = Num<float>::lt(a.v[0], dfloor) ? dfloor : a.v[0];
  const float rb = Num<float>::lt(b.v[0], dfloor) ? dfloor : b.v[0];
  const float ia = Num<float>::rcp(ra), ib = Num<float>::rcp(rb);
  PCell w;
  w.v[0] = make_float2(ra, rb);
#pragma unroll
  for (int v = 1; v < 4; ++v) w.v[v] = v < NV ? make_float2(__fmul_rn(ia, a.v[v]), __fmul_rn(ib, b.v[v])) : splat(0.f);
  return w;
}

// One column of a lane, both tiles: the primitives of rows j-3 .. j (PPM4's
// edges need only the cell itself, so the lean walk keeps 4 rows), the face
// value below row j-1, the upper edge of row j-3 and the y flux below row j-3.
struct Column2 {
  PCell W3, W2, W1, W0, Ay2, hy3, Fy3;
};

// Per tile of the pair: its origin, the lane's columns and where they go.
struct Half {
  int x0, y0, c0, gx[2], cx[2];
  bool out[2];
  bool real;  // false: a stand-in copy of tile A that computes and stores nothing of its own
};

__device__ __forceinline__ Half half_of(const StageParams& p, int tile, bool real, int lane) {
  Half h;
  const int bx = tile % p.tiles_x, by = tile / p.tiles_x;
  h.x0 = bx * kMarchTileX;
  h.y0 = by * p.ty;
  h.c0 = h.x0 - 3 + 2 * lane;
  h.real = real;
  const int xlast = min(h.x0 + kMarchTileX, p.nx) - 1;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    h.gx[k] = wrap_fast(h.c0 + k, p.nx);
    const int local = 2 * lane + k;
    h.out[k] = real && local >= 3 && local <= 60 && h.c0 + k < p.nx;
    h.cx[k] = min(max(h.c0 + k, h.x0), xlast);
  }
  return h;
}

// RK combine of one cell (the scalar kernel's, per half) and its CFL speeds.
template <int NV, bool BLEND>
__device__ __forceinline__ void combine_cell(const StageParams& p, const StageConsts<float>& k, const float* U,
                                             const float* V, float* Uo, float* Vo, size_t cell, bool store,
                                             const float (&w)[4], const float (&fl)[4], const float (&fr)[4],
                                             const float (&gl)[4], const float (&gr)[4], float ncx, float ncy,
                                             float& vmax0, float& vmax1) {
  using N = Num<float>;
  Cell4<float> u = load_cell<float, NV>(U + cell * NV);
  u.v[0] = w[0];  // the floored density
  Cell4<float> vs = load_cell<float, NV>(V + cell * NV);
  if (p.floor_v) vs.v[0] = N::lt(vs.v[0], k.dfloor) ? k.dfloor : vs.v[0];
  Cell4<float> un;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    if (p.has_delta) vs.v[v] = delta_update(vs.v[v], k.delta, u.v[v]);
    un.v[v] = rk_combine<float>(BLEND, k.g0, k.g1, u.v[v], vs.v[v], Ops<float>::sub(fr[v], fl[v]),
                                Ops<float>::sub(gr[v], gl[v]), ncx, ncy);
  }
  un.v[3] = NV == 4 ? un.v[3] : 0.f;
  if (p.floor_out) un.v[0] = N::lt(un.v[0], k.dfloor) ? k.dfloor : un.v[0];
  if (store) {
    if (p.has_delta && Vo) store_cell<float, NV>(Vo + cell * NV, vs);
    store_cell<float, NV>(Uo + cell * NV, un);
  }
  if (p.want_cfl) {
    const float inv = N::rcp(un.v[0]);
    const float s0 = signal_speed(inv, un.v[1], k.cs), s1 = signal_speed(inv, un.v[2], k.cs);
    if (store) {
      vmax0 = N::nanmax_pos(vmax0, s0);
      vmax1 = N::nanmax_pos(vmax1, s1);
    }
  }
}

template <int NV, bool BLEND>
__device__ __forceinline__ void march2_tiles(const StageParams& p, int tile_a, int tile_b, bool has_b, int ntiles) {
  const StageConsts<float>& k = stage_consts<float>(p);
  const int lane = threadIdx.x & 31;
  const int TY = p.ty;
  const Half A = half_of(p, tile_a, true, lane), B = half_of(p, has_b ? tile_b : tile_a, has_b, lane);
  const float* __restrict__ U = static_cast<const float*>(p.U);
  const float* __restrict__ V = static_cast<const float*>(p.V);
  float* Uo = static_cast<float*>(p.Uout);
  float* Vo = static_cast<float*>(p.Vout);
  Gas<float> gas;
  gas.cs = k.cs;
  gas.cs2 = k.cs2;
  gas.inv_cs = k.inv_cs;
  gas.half_inv_cs = k.half_inv_cs;
  gas.quarter_inv_cs = 0.5f * k.half_inv_cs;
  const float sdt = static_cast<float>(p.beta * p.clock->dt);
  const float ncx = -(sdt * k.inv_dx), ncy = -(sdt * k.inv_dy);

  Column2 col[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) col[h].W3 = col[h].W2 = col[h].W1 = col[h].W0 = col[h].Ay2 = col[h].hy3 = col[h].Fy3 = PCell{};
  float vmax[2][2] = {{0.f, 0.f}, {0.f, 0.f}};  // [tile][axis]
  const int iters = TY + 6;
  Cell4<float> na[2], nb[2];
  {
    const size_t ra = (size_t)wrap_fast(A.y0 - 3, p.ny) * p.nx, rb = (size_t)wrap_fast(B.y0 - 3, p.ny) * p.nx;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      na[h] = load_cell<float, NV>(U + (ra + A.gx[h]) * NV);
      nb[h] = load_cell<float, NV>(U + (rb + B.gx[h]) * NV);
    }
  }
  auto walk_row = [&](const int it, auto steady_tag) {
    constexpr bool kSteady = decltype(steady_tag)::value;
    const int ja = A.y0 - 3 + it, jb = B.y0 - 3 + it;
    PCell Ay1[2], lo[2], hi[2], Fy2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      Column2& c = col[h];
      c.W3 = c.W2;
      c.W2 = c.W1;
      c.W1 = c.W0;
      c.W0 = recover2<NV>(na[h], nb[h], k.dfloor);
    }
    {
      const size_t ra = (size_t)wrap_fast(ja + 1, p.ny) * p.nx, rb = (size_t)wrap_fast(jb + 1, p.ny) * p.nx;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        na[h] = load_cell<float, NV>(U + (ra + A.gx[h]) * NV);
        nb[h] = load_cell<float, NV>(U + (rb + B.gx[h]) * NV);
      }
    }
    // ---- y sweep --------------------------------------------------------------
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      Column2& c = col[h];
      Ay1[h] = c.Ay2;
      if (kSteady || it >= 3) Ay1[h] = faces2<NV>(c.W3, c.W2, c.W1, c.W0);
      hi[h] = c.hy3;
      lo[h] = c.hy3;
      if (kSteady || it >= 4) edges2<NV>(c.W2, c.Ay2, Ay1[h], lo[h], hi[h]);
      Fy2[h] = c.Fy3;
      if (kSteady || it >= 5) Fy2[h] = face_flux2<1, NV>(c.hy3, lo[h], gas);
    }
    if (kSteady) {
      // ---- x sweep of row r = j-3 across the lanes ------------------------------
      const PCell& a = col[0].W3;
      const PCell& b = col[1].W3;
      const PCell La = shfl_up<NV>(a, 1), Lb = shfl_up<NV>(b, 1);
      const PCell Ra = shfl_down<NV>(a, 1);  // PPM4's edges need no farther neighbour
      const PCell A0 = faces2<NV>(La, Lb, a, b);  // face c0
      const PCell A1 = faces2<NV>(Lb, a, b, Ra);  // face c0+1
      const PCell A2 = shfl_down<NV>(A0, 1);      // face c0+2
      PCell lo0, hi0, lo1, hi1;
      edges2<NV>(a, A0, A1, lo0, hi0);
      edges2<NV>(b, A1, A2, lo1, hi1);
      const PCell hiL = shfl_up<NV>(hi1, 1);
      const PCell F0 = face_flux2<0, NV>(hiL, lo0, gas);
      const PCell F1 = face_flux2<0, NV>(hi0, lo1, gas);
      const PCell F2 = shfl_down<NV>(F0, 1);
      const int ra = ja - 3, rb = jb - 3;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const PCell& fl = h == 0 ? F0 : F1;
        const PCell& fr = h == 0 ? F1 : F2;
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          const Half& T = t == 0 ? A : B;
          const int r = t == 0 ? ra : rb;
          if (r >= p.ny) continue;  // the same for every lane of the warp
          float w[4], l[4], rr[4], gl[4], gr[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            w[v] = t == 0 ? col[h].W3.v[v].x : col[h].W3.v[v].y;
            l[v] = t == 0 ? fl.v[v].x : fl.v[v].y;
            rr[v] = t == 0 ? fr.v[v].x : fr.v[v].y;
            gl[v] = t == 0 ? col[h].Fy3.v[v].x : col[h].Fy3.v[v].y;
            gr[v] = t == 0 ? Fy2[h].v[v].x : Fy2[h].v[v].y;
          }
          combine_cell<NV, BLEND>(p, k, U, V, Uo, Vo, (size_t)r * p.nx + (size_t)T.cx[h], T.out[h], w, l, rr, gl,
                                  gr, ncx, ncy, vmax[t][0], vmax[t][1]);
        }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      col[h].Ay2 = Ay1[h];
      col[h].hy3 = hi[h];
      col[h].Fy3 = Fy2[h];
    }
  };
  for (int it = 0; it < 6; ++it) walk_row(it, Flag<false>{});
#pragma unroll 1
  for (int it = 6; it < iters; ++it) walk_row(it, Flag<true>{});
  if (p.want_cfl) {
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const double m0 = warp_nan_max(static_cast<double>(vmax[t][0]));
      const double m1 = warp_nan_max(static_cast<double>(vmax[t][1]));
      const int tile = t == 0 ? tile_a : tile_b;
      if (lane == 0 && (t == 0 || has_b)) {
        p.partials[(size_t)tile * kCflSlots + 0] = m0;
        p.partials[(size_t)tile * kCflSlots + 1] = m1;
        p.partials[(size_t)tile * kCflSlots + 2] = 0.0;
        if (tile == 0) p.header->n_cfl = ntiles;
      }
    }
  }
}

}  // namespace pk

// Warp w walks tiles w and w + ceil(ntiles / 2); the block is one warp.
// Registers: two tiles' windows (112 values) plus temporaries, without
// spills: 4 variables take 232 registers (8 warps per SM), 3 variables fit
// 204 (10 warps); each warp does two tiles' work per instruction.
template <int NV, bool BLEND>
__global__ void __launch_bounds__(32, NV == 4 ? 8 : 10) stage_kernel_march_pairs(const StageParams p, int ntiles) {
  if (p.clock->done) return;
  const int half = (ntiles + 1) / 2;
  const int w = blockIdx.x;
  if (w >= half) return;
  const int b = w + half;
  pk::march2_tiles<NV, BLEND>(p, w, b, b < ntiles, ntiles);
}

template <int NV>
cudaError_t launch_march_pairs(const StageParams& p, int ntiles, bool blend, cudaStream_t s) {
  const int warps = (ntiles + 1) / 2;
  if (blend) stage_kernel_march_pairs<NV, true><<<warps, 32, 0, s>>>(p, ntiles);
  else stage_kernel_march_pairs<NV, false><<<warps, 32, 0, s>>>(p, ntiles);
  return cudaGetLastError();
}

}  // namespace jx
