// Float32 marching stage (DC, PLM, PPM4, PPMX or WENO-Z edges, any Riemann solver,
// the inviscid "lean" forms, 3 or 4 variables, two columns per lane) with the
// lane's two columns held as float32 pairs. Which (reconstruction, solver,
// variables, tile) combinations use it is decided by measurement; see
// march_packed in jx_stage_march.cuh.
//
// The marching kernel is bound by instruction issue. Its lane holds columns
// c0 and c0 + 1 of a 64-column strip and applies the same per-column
// arithmetic to both; here every value of the walk is a float2 (column c0's,
// column c0 + 1's) and every add, multiply and FMA of both sweeps is one
// packed Blackwell instruction (__fadd2_rn, __fmul2_rn, __ffma2_rn) for the
// two columns. Comparisons, selects, min/max, the SFU reciprocal and root,
// primitive recovery and the RK combine stay per column. The y sweep pairs
// directly (each column's window, face value, edges and flux); the x sweep
// pairs the two faces and two Riemann problems of the lane, whose operands
// are built from the lane's pair and its neighbours' by register moves.
//
// Each packed operation rounds each half exactly as the corresponding
// explicitly rounded float32 operation of jx_device.cuh (a - b is formed as
// fma(b, -1, a), which rounds once, as a - b does), so the results are the
// same bits as every other float32 stage kernel's (tested).
#pragma once
#include "jx_device.cuh"
#include "jx_internal.h"
#include "jx_ring.cuh"
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

// The lane's two columns of one cell-sized quantity (component v: column
// c0's in .x, column c0 + 1's in .y).
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

// (a's column c0 + 1, b's column c0): the pair one column to the right of a.
template <int NV>
__device__ __forceinline__ PCell straddle(const PCell& a, const PCell& b) {
  PCell o;
#pragma unroll
  for (int v = 0; v < 4; ++v) o.v[v] = v < NV ? make_float2(a.v[v].y, b.v[v].x) : splat(0.f);
  return o;
}

// (a's column c0 + 1, s): a's second half next to a per-column value.
template <int NV>
__device__ __forceinline__ PCell straddle(const PCell& a, const float (&s)[4]) {
  PCell o;
#pragma unroll
  for (int v = 0; v < 4; ++v) o.v[v] = v < NV ? make_float2(a.v[v].y, s[v]) : splat(0.f);
  return o;
}

// (s, a's column c0).
template <int NV>
__device__ __forceinline__ PCell straddle(const float (&s)[4], const PCell& a) {
  PCell o;
#pragma unroll
  for (int v = 0; v < 4; ++v) o.v[v] = v < NV ? make_float2(s[v], a.v[v].x) : splat(0.f);
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

// flux_roe_f32 for both halves (fluxes.py:134-172).
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

// flux_llf (float32 branch) for both halves (fluxes.py:175-183).
__device__ __forceinline__ void llf2(F2 dl, F2 dr, F2 ul, F2 ur, F2 tl, F2 tr, const Gas<float>& g, F2& f0, F2& f1,
                                     F2& f2) {
  const F2 cs = splat(g.cs), half = splat(0.5f);
  const F2 ml = mul(dl, ul), mr = mul(dr, ur);
  const F2 ql = mul(dl, tl), qr = mul(dr, tr);
  const F2 s0 = add(ml, mr);
  const F2 s1 = fma(ml, ul, fma(mr, ur, mul(splat(g.cs2), add(dl, dr))));
  const F2 s2 = fma(ml, tl, mul(mr, tr));
  const F2 nsp = neg(max2(add(abs2(ul), cs), add(abs2(ur), cs)));
  f0 = mul(half, fma(nsp, sub(dr, dl), s0));
  f1 = mul(half, fma(nsp, sub(mr, ml), s1));
  f2 = mul(half, fma(nsp, sub(qr, ql), s2));
}

// flux_hlle (float32 branch) for both halves (fluxes.py:186-201).
__device__ __forceinline__ void hlle2(F2 dl, F2 dr, F2 ul, F2 ur, F2 tl, F2 tr, const Gas<float>& g, F2& f0, F2& f1,
                                      F2& f2) {
  const F2 cs = splat(g.cs), cs2 = splat(g.cs2), half = splat(0.5f);
  const F2 r = mul(root2(dl), root2(dr));
  const F2 u = mul(fma(r, ur, mul(dl, ul)), rcp2(add(dl, r)));
  const F2 alo = min2(sub(u, cs), sub(ul, cs));
  const F2 ahi = max2(add(u, cs), add(ur, cs));
  const F2 bm = sel(alo.x < 0.f, alo.y < 0.f, alo, splat(-1e-20f));
  const F2 bp = sel(ahi.x > 0.f, ahi.y > 0.f, ahi, splat(1e-20f));
  const F2 vl = sub(ul, bm), vr = sub(ur, bp);
  const F2 ml = mul(dl, ul), mr = mul(dr, ur);
  const F2 fl0 = mul(dl, vl), fl1 = fma(ml, vl, mul(cs2, dl)), fl2 = mul(mul(dl, tl), vl);
  const F2 fr0 = mul(dr, vr), fr1 = fma(mr, vr, mul(cs2, dr)), fr2 = mul(mul(dr, tr), vr);
  const F2 num = mul(half, add(bp, bm)), den = sub(bp, bm);
  const F2 w = make_float2(Num<float>::quick_div(num.x, den.x), Num<float>::quick_div(num.y, den.y));
  f0 = fma(w, sub(fl0, fr0), mul(half, add(fl0, fr0)));
  f1 = fma(w, sub(fl1, fr1), mul(half, add(fl1, fr1)));
  f2 = fma(w, sub(fl2, fr2), mul(half, add(fl2, fr2)));
}

// face_flux_cells for both halves: Riemann flux in x/y component order plus
// passive-scalar upwinding.
template <int RS, int DIR, int NV>
__device__ __forceinline__ PCell face_flux2(const PCell& L, const PCell& Rv, const Gas<float>& g) {
  constexpr int nn = DIR == 0 ? 1 : 2, tt = DIR == 0 ? 2 : 1;
  F2 f0, fn, ft;
  if constexpr (RS == JX_LLF) llf2(L.v[0], Rv.v[0], L.v[nn], Rv.v[nn], L.v[tt], Rv.v[tt], g, f0, fn, ft);
  else if constexpr (RS == JX_HLLE) hlle2(L.v[0], Rv.v[0], L.v[nn], Rv.v[nn], L.v[tt], Rv.v[tt], g, f0, fn, ft);
  else roe2(L.v[0], Rv.v[0], L.v[nn], Rv.v[nn], L.v[tt], Rv.v[tt], g, f0, fn, ft);
  PCell f;
  f.v[0] = f0;
  f.v[1] = DIR == 0 ? fn : ft;
  f.v[2] = DIR == 0 ? ft : fn;
  f.v[3] = splat(0.f);
#pragma unroll
  for (int v = 3; v < NV; ++v) f.v[v] = mul(f0, sel(f0.x >= 0.f, f0.y >= 0.f, L.v[v], Rv.v[v]));
  return f;
}


// -(c ? a : 0) per half (a negative zero where c is false, as the scalar form).
__device__ __forceinline__ F2 neg_if(bool cx, bool cy, F2 a) { return make_float2(-(cx ? a.x : 0.f), -(cy ? a.y : 0.f)); }

// ppmx_edge (float32) for both halves: the smooth-extremum limiter of one
// face value (fluxes.py:45-53).
__device__ __forceinline__ F2 ppmx_edge2(F2 a, F2 b, F2 edge, F2 ca, F2 cb) {
  using N = Num<float>;
  const F2 curv = mul(splat(3.f), fma(splat(-2.f), edge, add(a, b)));
  const bool ax = (curv.x > 0.f && ca.x > 0.f && cb.x > 0.f) || (curv.x < 0.f && ca.x < 0.f && cb.x < 0.f);
  const bool ay = (curv.y > 0.f && ca.y > 0.f && cb.y > 0.f) || (curv.y < 0.f && ca.y < 0.f && cb.y < 0.f);
  const F2 mag = make_float2(N::pmin(fabsf(ca.x), fabsf(cb.x)), N::pmin(fabsf(ca.y), fabsf(cb.y)));
  const F2 m125 = mul(splat(1.25f), mag);
  const F2 lim = make_float2(copysignf(N::pmin(m125.x, fabsf(curv.x)), curv.x),
                             copysignf(N::pmin(m125.y, fabsf(curv.y)), curv.y));
  const F2 fixed = fma(neg_if(ax, ay, lim), splat(float(1.0 / 6.0)), mul(splat(0.5f), add(a, b)));
  const F2 p = mul(sub(a, edge), sub(b, edge));
  return sel(p.x > 0.f, p.y > 0.f, fixed, edge);
}

// ppmx_face (float32) for both halves (fluxes.py:62-68).
__device__ __forceinline__ F2 ppmx_face2(F2 w0, F2 w1, F2 w2, F2 w3) {
  const F2 e = mul(fma(splat(7.f), add(w2, w1), neg(add(w0, w3))), splat(float(1.0 / 12.0)));
  const F2 c1 = fma(splat(-2.f), w1, add(w0, w2));
  const F2 c2 = fma(splat(-2.f), w2, add(w1, w3));
  return ppmx_edge2(w1, w2, e, c1, c2);
}

// ppmx_cell (float32 branch) for both halves (fluxes.py:70-84).
__device__ __forceinline__ void ppmx_cell2(F2 m2, F2 m1, F2 c, F2 p1, F2 p2, F2 lo_face, F2 hi_face, F2& lo, F2& hi) {
  using N = Num<float>;
  const F2 cl = fma(splat(-2.f), m1, add(m2, c));
  const F2 cm = fma(splat(-2.f), c, add(m1, p1));
  const F2 cr = fma(splat(-2.f), p1, add(c, p2));
  const F2 dh = sub(hi_face, c);
  const F2 dl = sub(lo_face, c);
  const F2 e1 = mul(dh, sub(c, lo_face)), e2 = mul(sub(m1, c), sub(c, p1));
  const bool ext_x = e1.x <= 0.f || e2.x <= 0.f, ext_y = e1.y <= 0.f || e2.y <= 0.f;
  const F2 d2 = mul(splat(6.f), fma(splat(-2.f), c, add(lo_face, hi_face)));
  const bool ag_x = (d2.x > 0.f && cl.x > 0.f && cm.x > 0.f && cr.x > 0.f) ||
                    (d2.x < 0.f && cl.x < 0.f && cm.x < 0.f && cr.x < 0.f);
  const bool ag_y = (d2.y > 0.f && cl.y > 0.f && cm.y > 0.f && cr.y > 0.f) ||
                    (d2.y < 0.f && cl.y < 0.f && cm.y < 0.f && cr.y < 0.f);
  const F2 mag = make_float2(N::pmin(fabsf(cm.x), N::pmin(fabsf(cl.x), fabsf(cr.x))),
                             N::pmin(fabsf(cm.y), N::pmin(fabsf(cl.y), fabsf(cr.y))));
  const F2 m125 = mul(splat(1.25f), mag);
  const F2 lim = make_float2(copysignf(N::pmin(m125.x, fabsf(d2.x)), d2.x),
                             copysignf(N::pmin(m125.y, fabsf(d2.y)), d2.y));
  const F2 scale = make_float2(N::pmax(fabsf(m1.x), N::pmax(fabsf(c.x), fabsf(p1.x))),
                               N::pmax(fabsf(m1.y), N::pmax(fabsf(c.y), fabsf(p1.y))));
  const F2 thr = mul(splat(float(1e-12)), scale);
  const bool use_x = ag_x && fabsf(d2.x) > thr.x, use_y = ag_y && fabsf(d2.y) > thr.y;
  const F2 ratio = make_float2(use_x ? N::quick_div(lim.x, d2.x) : 0.f, use_y ? N::quick_div(lim.y, d2.y) : 0.f);
  const bool slo_x = fabsf(dl.x) >= 2.f * fabsf(dh.x), slo_y = fabsf(dl.y) >= 2.f * fabsf(dh.y);
  const bool shi_x = fabsf(dh.x) >= 2.f * fabsf(dl.x), shi_y = fabsf(dh.y) >= 2.f * fabsf(dl.y);
  const F2 lm = sel(slo_x, slo_y, fma(splat(-2.f), dh, c), lo_face);
  const F2 hm = sel(shi_x, shi_y, fma(splat(-2.f), dl, c), hi_face);
  lo = sel(ext_x, ext_y, fma(dl, ratio, c), lm);
  hi = sel(ext_x, ext_y, fma(dh, ratio, c), hm);
}

__device__ __forceinline__ F2 div2(F2 a, F2 b) { return make_float2(Num<float>::div(a.x, b.x), Num<float>::div(a.y, b.y)); }

// plm_cell (float32) for both halves (fluxes.py:11-18, harmonic-mean slope).
__device__ __forceinline__ void plm_cell2(F2 m1, F2 c, F2 p1, F2& lo, F2& hi) {
  const F2 bw = sub(c, m1), fw = sub(p1, c);
  const F2 p = mul(bw, fw), s = add(bw, fw);
  const F2 hs = make_float2(p.x > 0.f ? Num<float>::quick_div(p.x, s.x) : 0.f,
                            p.y > 0.f ? Num<float>::quick_div(p.y, s.y) : 0.f);
  hi = add(c, hs);
  lo = sub(c, hs);
}

// wenoz_combine (float32) for both halves (fluxes.py:87-93).
__device__ __forceinline__ F2 wenoz_combine2(F2 s0, F2 s1, F2 s2, F2 s3, F2 s4, F2 w0, F2 w1, F2 w2) {
  const F2 a0 = mul(splat(0.1f), w0), a1 = mul(splat(0.6f), w1), a2 = mul(splat(0.3f), w2);
  const F2 f0 = fma(splat(11.f), s2, fma(splat(-7.f), s1, mul(splat(2.f), s0)));
  const F2 f1 = fma(splat(2.f), s3, fma(splat(5.f), s2, neg(s1)));
  const F2 f2 = sub(fma(splat(5.f), s3, mul(splat(2.f), s2)), s4);
  const F2 num = fma(f2, a2, fma(f1, a1, mul(f0, a0)));
  return div2(num, mul(splat(6.f), add(add(a0, a1), a2)));
}

// wenoz_cell_f32 for both halves (fluxes.py:96-117).
__device__ __forceinline__ void wenoz_cell2(F2 m2, F2 m1, F2 c, F2 p1, F2 p2, F2& lo, F2& hi) {
  const F2 k1312 = splat(float(13.0 / 12.0)), q = splat(0.25f);
  const F2 eps = splat(1e-42f > Tiny<float>::value ? 1e-42f : Tiny<float>::value);
  const F2 t0 = fma(splat(-2.f), m1, add(m2, c)), u0 = fma(splat(-4.f), m1, fma(splat(3.f), c, m2));
  const F2 t1 = fma(splat(-2.f), c, add(m1, p1)), u1 = sub(m1, p1);
  const F2 t2 = fma(splat(-2.f), p1, add(p2, c)), u2 = fma(splat(-4.f), p1, fma(splat(3.f), c, p2));
  const F2 b0 = fma(k1312, mul(t0, t0), mul(q, mul(u0, u0)));
  const F2 b1 = fma(k1312, mul(t1, t1), mul(q, mul(u1, u1)));
  const F2 b2 = fma(k1312, mul(t2, t2), mul(q, mul(u2, u2)));
  const F2 tau = abs2(sub(b0, b2));
  const F2 d0 = add(b0, eps), d1 = add(b1, eps), d2 = add(b2, eps);
  const F2 dmin = min2(d0, min2(d1, d2));
  const F2 inv_sc = div2(splat(1.f), max2(tau, dmin));
  F2 base = mul(dmin, inv_sc);
  base = mul(base, base);
  const F2 con = mul(tau, inv_sc);
  const F2 r0 = mul(con, div2(dmin, d0)), r1 = mul(con, div2(dmin, d1)), r2 = mul(con, div2(dmin, d2));
  const F2 w0 = fma(r0, r0, base), w1 = fma(r1, r1, base), w2 = fma(r2, r2, base);
  hi = wenoz_combine2(m2, m1, c, p1, p2, w0, w1, w2);
  lo = wenoz_combine2(p2, p1, c, m1, m2, w2, w1, w0);
}

template <int RECON, int NV>
__device__ __forceinline__ PCell faces2(const PCell& w0, const PCell& w1, const PCell& w2, const PCell& w3) {
  PCell a;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    if (v >= NV) a.v[v] = splat(0.f);
    else if constexpr (RECON == JX_PPM4) a.v[v] = ppm4_face2(w0.v[v], w1.v[v], w2.v[v], w3.v[v]);
    else a.v[v] = ppmx_face2(w0.v[v], w1.v[v], w2.v[v], w3.v[v]);
  }
  return a;
}

// edges_cells for both halves: the low/high edges of the cells at the
// centre of (m2, m1, c, p1, p2); lf/hf the face values (PPM4 only).
template <int RECON, int NV>
__device__ __forceinline__ void edges2(const PCell& m2, const PCell& m1, const PCell& c, const PCell& p1,
                                       const PCell& p2, const PCell& lf, const PCell& hf, float dfloor, PCell& lo,
                                       PCell& hi) {
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    if (v < NV) {
      if constexpr (RECON == JX_DC) {
        lo.v[v] = hi.v[v] = c.v[v];
      } else if constexpr (RECON == JX_PLM) {
        plm_cell2(m1.v[v], c.v[v], p1.v[v], lo.v[v], hi.v[v]);
      } else if constexpr (RECON == JX_PPM4) {
        ppm4_cell2(c.v[v], lf.v[v], hf.v[v], lo.v[v], hi.v[v]);
      } else if constexpr (RECON == JX_PPMX) {
        ppmx_cell2(m2.v[v], m1.v[v], c.v[v], p1.v[v], p2.v[v], lf.v[v], hf.v[v], lo.v[v], hi.v[v]);
      } else {
        wenoz_cell2(m2.v[v], m1.v[v], c.v[v], p1.v[v], p2.v[v], lo.v[v], hi.v[v]);
      }
    } else {
      lo.v[v] = hi.v[v] = splat(0.f);
    }
  }
  if constexpr (RECON == JX_PPMX || RECON == JX_WENOZ) {  // fluxes.py:128-130
    lo.v[0] = max2(lo.v[0], splat(dfloor));
    hi.v[0] = max2(hi.v[0], splat(dfloor));
  }
}

// The lane's two cells (columns c0 and c0 + 1) recovered into a pair: the
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

// viscous_face (float32 branch) for both halves (fluxes.py:227-266): the
// momentum flux of the face between cells a (low side) and b (high side)
// from their velocities and the transverse sums (tp: columns or rows on the
// high side, tm: on the low side).
template <int DIR>
__device__ __forceinline__ void viscous_face2(bool smag, float nu0, float smag_c, float inv_dn, float inv_4dt,
                                              F2 rho_a, F2 rho_b, F2 ax, F2 ay, F2 bx, F2 by, F2 tpx, F2 tpy,
                                              F2 tmx, F2 tmy, F2& f1, F2& f2) {
  const F2 dn_x = mul(sub(bx, ax), splat(inv_dn)), dn_y = mul(sub(by, ay), splat(inv_dn));
  const F2 dt_x = mul(sub(tpx, tmx), splat(inv_4dt)), dt_y = mul(sub(tpy, tmy), splat(inv_4dt));
  const F2 dvx_dx = DIR == 0 ? dn_x : dt_x, dvy_dx = DIR == 0 ? dn_y : dt_y;
  const F2 dvx_dy = DIR == 0 ? dt_x : dn_x, dvy_dy = DIR == 0 ? dt_y : dn_y;
  const F2 shear = add(dvy_dx, dvx_dy);
  const F2 k43 = splat(float(4.0 / 3.0)), k23 = splat(float(2.0 / 3.0));
  const F2 s0 = DIR == 0 ? fma(k43, dvx_dx, neg(mul(k23, dvy_dy))) : shear;
  const F2 s1 = DIR == 0 ? shear : fma(k43, dvy_dy, neg(mul(k23, dvx_dx)));
  F2 nu = splat(nu0);
  if (smag) {
    const F2 s2 = fma(shear, shear, mul(splat(2.f), fma(dvx_dx, dvx_dx, mul(dvy_dy, dvy_dy))));
    nu = fma(splat(smag_c), make_float2(sqrtf(s2.x), sqrtf(s2.y)), nu);
  }
  const F2 mu = neg(mul(mul(splat(0.5f), nu), add(rho_b, rho_a)));
  f1 = fma(mu, s0, f1);
  f2 = fma(mu, s1, f2);
}

// The lane's columns: the primitives of rows j-4 .. j (only WENO-Z reads
// row j-4), the face value below row j-1 (PPM4), the upper edge of row j-3
// and the y flux below row j-3.
struct ColumnPair {
  PCell W4, W3, W2, W1, W0, Ay2, hy3, Fy3;
};

// One tile of kMarchTileX (58) columns by p.ty rows, one warp, two columns
// per lane (lane l: columns c0 = x0 - 3 + 2 l and c0 + 1), as march_tile in
// jx_stage_march.cuh walks it, with the same row ring when RING.
// FORM: 0 = generic (viscosity, Smagorinsky, drag and the blend flag read at
// run time; no SGS stress), 1 = lean plain, 2 = lean blend (the MarchForm
// values).
// XFIRST: run each row's x sweep ahead of its y sweep (fewer values live
// across the row: the single-solve PPM4 ring kernel fits 112 registers
// without spills only this way). Either order gives the same bits.
template <int RECON, int RS, int NV, int FORM, bool RING, bool XFIRST = false>
__device__ __forceinline__ void march_tile_pk(const StageParams& p, int tile, int ntiles, float4* ring) {
  using N = Num<float>;
  const StageConsts<float>& k = stage_consts<float>(p);
  const int lane = threadIdx.x & 31;
  const int TY = p.ty;
  const int bx = tile % p.tiles_x, by = tile / p.tiles_x;
  const int x0 = bx * kMarchTileX;
  const int y0 = by * TY;
  const int c0 = x0 - 3 + 2 * lane;
  const int xlast = min(x0 + kMarchTileX, p.nx) - 1;
  int gx[2], cx[2];
  bool out[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    gx[h] = wrap_fast(c0 + h, p.nx);
    const int local = 2 * lane + h;
    out[h] = local >= 3 && local <= 60 && c0 + h < p.nx;
    cx[h] = min(max(c0 + h, x0), xlast);
  }
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
  constexpr bool kLean = FORM != 0;
  const bool visc = !kLean && p.visc_on;
  const bool drag = !kLean && p.drag_on;
  const bool blend = kLean ? FORM == 2 : (bool)p.blend;
  const float kdrag = sdt * k.drag;
  constexpr unsigned kAll = 0xffffffffu;

  ColumnPair c;
  c.W4 = c.W3 = c.W2 = c.W1 = c.W0 = c.Ay2 = c.hy3 = c.Fy3 = PCell{};
  float vmax0 = 0.f, vmax1 = 0.f;
  const int iters = TY + 6;
  Cell4<float> next[2];
  auto ringU = [&](int t, int h) { return ring + ((t & (kRingU - 1)) * 2 + h) * 32 + lane; };
  auto ringV = [&](int t, int h) { return ring + (kRingU * 2 + (t & (kRingV - 1)) * 2 + h) * 32 + lane; };
  if constexpr (RING) {
    for (int t = 0; t < kRingAhead; ++t) {
      const size_t row = (size_t)wrap_fast(y0 - 3 + t, p.ny) * p.nx;
#pragma unroll
      for (int h = 0; h < 2; ++h) ring_copy<NV>(ringU(t, h), U + (row + gx[h]) * NV);
      cp_async_commit();
    }
  } else {
    const size_t row = (size_t)wrap_fast(y0 - 3, p.ny) * p.nx;
#pragma unroll
    for (int h = 0; h < 2; ++h) next[h] = load_cell<float, NV>(U + (row + gx[h]) * NV);
  }
  auto walk_row = [&](const int it, auto steady_tag) {
    constexpr bool kSteady = decltype(steady_tag)::value;
    const int j = y0 - 3 + it;
    if constexpr (RING) {
      // As in march_tile: this row's U and the V the combine reads (row
      // it - 3) came in group it of kRingAhead + it committed ones.
      cp_async_wait<kRingAhead - 1>();
#pragma unroll
      for (int h = 0; h < 2; ++h) next[h] = ring_read<NV>(ringU(it, h));
    }
    c.W4 = c.W3;
    c.W3 = c.W2;
    c.W2 = c.W1;
    c.W1 = c.W0;
    c.W0 = recover2<NV>(next[0], next[1], k.dfloor);
    if constexpr (RING) {
      if (it + kRingAhead < iters) {
        const size_t row = (size_t)wrap_fast(j + kRingAhead, p.ny) * p.nx;
#pragma unroll
        for (int h = 0; h < 2; ++h) ring_copy<NV>(ringU(it + kRingAhead, h), U + (row + gx[h]) * NV);
      }
      if (it >= 3 && j < p.ny && it < TY + 3) {
        const size_t row = (size_t)j * p.nx;
#pragma unroll
        for (int h = 0; h < 2; ++h) ring_copy<NV>(ringV(it, h), V + (row + (size_t)cx[h]) * NV);
      }
      cp_async_commit();
    } else {
      const size_t row = (size_t)wrap_fast(j + 1, p.ny) * p.nx;
#pragma unroll
      for (int h = 0; h < 2; ++h) next[h] = load_cell<float, NV>(U + (row + gx[h]) * NV);
    }
    // ---- x sweep of row r = j-3 across the lanes (dfx: the two cells' x flux
    // differences); with XFIRST ahead of the y sweep, else just before the
    // combine ---------------------------------------------------------------
    PCell dfx;
    auto x_sweep = [&] {
      const PCell& own = c.W3;                           // columns (c0, c0+1)
      const PCell L = shfl_up<NV>(own, 1);               // (c0-2, c0-1)
      const PCell R = shfl_down<NV>(own, 1);             // (c0+2, c0+3)
      const PCell m1 = straddle<NV>(L, own);             // (c0-1, c0)
      const PCell p1 = straddle<NV>(own, R);             // (c0+1, c0+2)
      PCell lf = own, hf = own;
      if constexpr (RECON == JX_PPM4 || RECON == JX_PPMX) {
        lf = faces2<RECON, NV>(L, m1, own, p1);  // faces c0, c0+1
        float A2[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) A2[v] = v < NV ? __shfl_down_sync(0xffffffffu, lf.v[v].x, 1) : 0.f;  // face c0+2
        hf = straddle<NV>(lf, A2);
      }
      float hiL[4], F2s[4];
      PCell lx, hx;
      edges2<RECON, NV>(L, m1, own, p1, R, lf, hf, k.dfloor, lx, hx);
#pragma unroll
      for (int v = 0; v < 4; ++v) hiL[v] = v < NV ? __shfl_up_sync(0xffffffffu, hx.v[v].y, 1) : 0.f;  // column c0-1
      PCell F01 = face_flux2<RS, 0, NV>(straddle<NV>(hiL, hx), lx, gas);  // fluxes at faces c0, c0+1
      if (visc) {
        // Transverse y sums at the faces' two columns: rows r+1 (W2) and r-1 (W4).
        const F2 ux = c.W2.v[1], uy = c.W2.v[2], dx = c.W4.v[1], dy = c.W4.v[2];
        const F2 uxm = make_float2(__shfl_up_sync(kAll, ux.y, 1), ux.x), uym = make_float2(__shfl_up_sync(kAll, uy.y, 1), uy.x);
        const F2 dxm = make_float2(__shfl_up_sync(kAll, dx.y, 1), dx.x), dym = make_float2(__shfl_up_sync(kAll, dy.y, 1), dy.x);
        viscous_face2<0>(p.smag_on, k.nu, k.smag_c, k.inv_dx, k.inv_4dy, m1.v[0], own.v[0], m1.v[1], m1.v[2],
                         own.v[1], own.v[2], add(ux, uxm), add(uy, uym), add(dx, dxm), add(dy, dym), F01.v[1],
                         F01.v[2]);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) F2s[v] = v < NV ? __shfl_down_sync(0xffffffffu, F01.v[v].x, 1) : 0.f;  // face c0+2
      // The flux differences of both cells, each rounded on its own.
      const PCell F12 = straddle<NV>(F01, F2s);
#pragma unroll
      for (int v = 0; v < 4; ++v) dfx.v[v] = sub(F12.v[v], F01.v[v]);
    };
    if constexpr (XFIRST)
      if (kSteady) x_sweep();
    // ---- y sweep of both columns -------------------------------------------
    PCell Ay1 = c.Ay2;
    if constexpr (RECON == JX_PPM4 || RECON == JX_PPMX)
      if (kSteady || it >= 3) Ay1 = faces2<RECON, NV>(c.W3, c.W2, c.W1, c.W0);
    PCell lo = c.hy3, hi = c.hy3;
    if (kSteady || it >= 4) edges2<RECON, NV>(c.W4, c.W3, c.W2, c.W1, c.W0, c.Ay2, Ay1, k.dfloor, lo, hi);
    PCell Fy2 = c.Fy3;
    if (kSteady || it >= 5) {
      Fy2 = face_flux2<RS, 1, NV>(c.hy3, lo, gas);
      if (visc) {
        // Transverse x sums (row j-2 + row j-3) at the columns either side;
        // a neighbour lane's sum is the same number it formed itself.
        const F2 Sx = add(c.W2.v[1], c.W3.v[1]), Sy = add(c.W2.v[2], c.W3.v[2]);
        const float sxm = __shfl_up_sync(kAll, Sx.y, 1), sym = __shfl_up_sync(kAll, Sy.y, 1);      // column c0-1
        const float sxp = __shfl_down_sync(kAll, Sx.x, 1), syp = __shfl_down_sync(kAll, Sy.x, 1);  // column c0+2
        viscous_face2<1>(p.smag_on, k.nu, k.smag_c, k.inv_dy, k.inv_4dx, c.W3.v[0], c.W2.v[0], c.W3.v[1], c.W3.v[2],
                         c.W2.v[1], c.W2.v[2], make_float2(Sx.y, sxp), make_float2(Sy.y, syp),
                         make_float2(sxm, Sx.x), make_float2(sym, Sy.x), Fy2.v[1], Fy2.v[2]);
      }
    }
    if (kSteady) {
      if constexpr (!XFIRST) x_sweep();
      const PCell& own = c.W3;
      PCell dfy;
#pragma unroll
      for (int v = 0; v < 4; ++v) dfy.v[v] = sub(Fy2.v[v], c.Fy3.v[v]);
      const int r = j - 3;
      if (r < p.ny) {
        const size_t row = (size_t)r * p.nx;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const size_t cell = row + (size_t)cx[h];
          Cell4<float> u, vs;
          if constexpr (RING) {
            u = ring_read<NV>(ringU(it - 3, h));
            vs = ring_read<NV>(ringV(it - 3, h));
          } else {
            u = load_cell<float, NV>(U + cell * NV);
            vs = load_cell<float, NV>(V + cell * NV);
          }
          u.v[0] = h == 0 ? own.v[0].x : own.v[0].y;  // the floored density
          if (p.floor_v) vs.v[0] = N::lt(vs.v[0], k.dfloor) ? k.dfloor : vs.v[0];
          Cell4<float> un;
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            if (p.has_delta) vs.v[v] = delta_update(vs.v[v], k.delta, u.v[v]);
            un.v[v] = rk_combine<float>(blend, k.g0, k.g1, u.v[v], vs.v[v], h == 0 ? dfx.v[v].x : dfx.v[v].y,
                                        h == 0 ? dfy.v[v].x : dfy.v[v].y, ncx, ncy);
          }
          un.v[3] = NV == 4 ? un.v[3] : 0.f;
          if (drag) {
            const float w0 = h == 0 ? own.v[0].x : own.v[0].y;
            un.v[1] = drag_term(un.v[1], kdrag * w0, h == 0 ? own.v[1].x : own.v[1].y);
            un.v[2] = drag_term(un.v[2], kdrag * w0, h == 0 ? own.v[2].x : own.v[2].y);
          }
          if (p.floor_out) un.v[0] = N::lt(un.v[0], k.dfloor) ? k.dfloor : un.v[0];
          if (out[h]) {
            if (p.has_delta && Vo) store_cell<float, NV>(Vo + cell * NV, vs);
            store_cell<float, NV>(Uo + cell * NV, un);
          }
          if (p.want_cfl) {
            const float inv = N::rcp(un.v[0]);
            const float s0 = signal_speed(inv, un.v[1], k.cs), s1 = signal_speed(inv, un.v[2], k.cs);
            if (out[h]) {
              vmax0 = N::nanmax_pos(vmax0, s0);
              vmax1 = N::nanmax_pos(vmax1, s1);
            }
          }
        }
      }
    }
    c.Ay2 = Ay1;
    c.hy3 = hi;
    c.Fy3 = Fy2;
  };
  for (int it = 0; it < 6; ++it) walk_row(it, Flag<false>{});
#pragma unroll 1
  for (int it = 6; it < iters; ++it) walk_row(it, Flag<true>{});
  if constexpr (RING) cp_async_wait_all();
  if (p.want_cfl) {
    const double m0 = warp_nan_max(static_cast<double>(vmax0));
    const double m1 = warp_nan_max(static_cast<double>(vmax1));
    if (lane == 0) {
      p.partials[(size_t)tile * kCflSlots + 0] = m0;
      p.partials[(size_t)tile * kCflSlots + 1] = m1;
      p.partials[(size_t)tile * kCflSlots + 2] = 0.0;
      if (tile == 0) p.header->n_cfl = ntiles;
    }
  }
}

}  // namespace pk
}  // namespace jx
