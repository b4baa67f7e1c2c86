// Device-side building blocks of the fused isothermal stage kernel:
// per-cell edge reconstructions, Riemann solvers, NaN-propagating min/max
// and block reductions. Arithmetic follows the reference's operation order
// (jathenax/fluxes.py), with two deliberate changes that the FP64 parity
// tolerance (1e-12 relative per stage) covers: divisions by loop-invariant
// constants (12, 6, cs, dx, dy) become multiplications by the reciprocal,
// and nvcc contracts a*b+c into FMA.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace jx {

template <typename R> struct Tiny;
template <> struct Tiny<double> { static constexpr double value = 2.2250738585072014e-308; };
template <> struct Tiny<float> { static constexpr float value = 1.17549435e-38f; };

// max/min that return NaN when either argument is NaN (jnp.maximum/minimum,
// and jnp.max/min reductions), unlike fmax/fmin.
template <typename T> __device__ __forceinline__ T nan_max(T a, T b) {
  return (a > b || a != a) ? a : b;
}
template <typename T> __device__ __forceinline__ T nan_min(T a, T b) {
  return (a < b || a != a) ? a : b;
}

// ---------------------------------------------------------------------------
// Reconstructions: (m2, m1, c, p1, p2) are one primitive at cells i-2..i+2;
// produce the limited values at the low (lo) and high (hi) edges of cell i.
// The face between cells i-1 and i takes left = hi(i-1), right = lo(i).
// ---------------------------------------------------------------------------

template <typename R>
__device__ __forceinline__ void edges_dc(R, R, R c, R, R, R& lo, R& hi) {
  lo = c;  // fluxes.py:6-8
  hi = c;
}

template <typename R>
__device__ __forceinline__ void edges_plm(R, R m1, R c, R p1, R, R& lo, R& hi) {
  // fluxes.py:11-18, harmonic-mean slope.
  R bw = c - m1;
  R fw = p1 - c;
  R prod = bw * fw;
  R hs = prod > R(0) ? prod / (bw + fw) : R(0);
  hi = c + hs;
  lo = c - hs;
}

template <typename R>
__device__ __forceinline__ void edges_ppm4(R m2, R m1, R c, R p1, R p2, R& lo, R& hi) {
  // fluxes.py:21-42.
  const R k12 = R(1.0 / 12.0);
  R l = (R(7) * (c + m1) - (m2 + p1)) * k12;
  R h = (R(7) * (c + p1) - (m1 + p2)) * k12;
  l = fmin(fmax(l, fmin(c, m1)), fmax(c, m1));
  h = fmin(fmax(h, fmin(c, p1)), fmax(c, p1));
  R dh = h - c;
  R dl = l - c;
  bool flat = dh * dl >= R(0);
  R l2 = fabs(dl) >= R(2) * fabs(dh) ? c - R(2) * dh : l;
  R h2 = fabs(dh) >= R(2) * fabs(dl) ? c - R(2) * dl : h;
  lo = flat ? c : l2;
  hi = flat ? c : h2;
}

template <typename R>
__device__ __forceinline__ R ppmx_edge(R a, R b, R edge, R ca, R cb) {
  // fluxes.py:45-53.
  R curv = R(3) * ((a + b) - R(2) * edge);
  bool agree = (curv > R(0) && ca > R(0) && cb > R(0)) || (curv < R(0) && ca < R(0) && cb < R(0));
  R mag = fmin(fabs(ca), fabs(cb));
  R lim = copysign(fmin(R(1.25) * mag, fabs(curv)), curv);
  R fixed = R(0.5) * (a + b) - (agree ? lim : R(0)) * R(1.0 / 6.0);
  return (a - edge) * (b - edge) > R(0) ? fixed : edge;
}

template <typename R>
__device__ __forceinline__ void edges_ppmx(R m2, R m1, R c, R p1, R p2, R& lo, R& hi) {
  // fluxes.py:56-84.
  const R k12 = R(1.0 / 12.0);
  R l = (R(7) * (c + m1) - (m2 + p1)) * k12;
  R h = (R(7) * (c + p1) - (m1 + p2)) * k12;
  R cl = (m2 + c) - R(2) * m1;
  R cm = (m1 + p1) - R(2) * c;
  R cr = (c + p2) - R(2) * p1;
  l = ppmx_edge(m1, c, l, cl, cm);
  h = ppmx_edge(c, p1, h, cm, cr);
  R dh = h - c;
  R dl = l - c;
  bool ext = (dh * (c - l) <= R(0)) || ((m1 - c) * (c - p1) <= R(0));
  R d2 = R(6) * ((l + h) - R(2) * c);
  bool agree = (d2 > R(0) && cl > R(0) && cm > R(0) && cr > R(0)) ||
               (d2 < R(0) && cl < R(0) && cm < R(0) && cr < R(0));
  R mag = fmin(fabs(cm), fmin(fabs(cl), fabs(cr)));
  R lim = copysign(fmin(R(1.25) * mag, fabs(d2)), d2);
  R scale = fmax(fabs(m1), fmax(fabs(c), fabs(p1)));
  bool use = agree && (fabs(d2) > R(1e-12) * scale);
  R ratio = use ? lim / d2 : R(0);
  R lm = fabs(dl) >= R(2) * fabs(dh) ? c - R(2) * dh : l;
  R hm = fabs(dh) >= R(2) * fabs(dl) ? c - R(2) * dl : h;
  lo = ext ? c + dl * ratio : lm;
  hi = ext ? c + dh * ratio : hm;
}

template <typename R>
__device__ __forceinline__ R wenoz_combine(R s0, R s1, R s2, R s3, R s4, R w0, R w1, R w2) {
  // fluxes.py:87-93.
  R a0 = R(0.1) * w0, a1 = R(0.6) * w1, a2 = R(0.3) * w2;
  R f0 = R(2) * s0 - R(7) * s1 + R(11) * s2;
  R f1 = -s1 + R(5) * s2 + R(2) * s3;
  R f2 = R(2) * s2 + R(5) * s3 - s4;
  return (f0 * a0 + f1 * a1 + f2 * a2) / (R(6) * (a0 + a1 + a2));
}

template <typename R>
__device__ __forceinline__ void edges_wenoz(R m2, R m1, R c, R p1, R p2, R& lo, R& hi) {
  // fluxes.py:96-117; eps = max(1e-42, finfo(dtype).tiny) at fluxes.py:108.
  const R k1312 = R(13.0 / 12.0);
  const R eps = R(1e-42) > Tiny<R>::value ? R(1e-42) : Tiny<R>::value;
  R t0 = (m2 + c) - R(2) * m1, u0 = (m2 + R(3) * c) - R(4) * m1;
  R t1 = (m1 + p1) - R(2) * c, u1 = m1 - p1;
  R t2 = (p2 + c) - R(2) * p1, u2 = (p2 + R(3) * c) - R(4) * p1;
  R b0 = k1312 * (t0 * t0) + R(0.25) * (u0 * u0);
  R b1 = k1312 * (t1 * t1) + R(0.25) * (u1 * u1);
  R b2 = k1312 * (t2 * t2) + R(0.25) * (u2 * u2);
  R tau = fabs(b0 - b2);
  R d0 = b0 + eps, d1 = b1 + eps, d2 = b2 + eps;
  R dmin = fmin(d0, fmin(d1, d2));
  R inv_sc = R(1) / fmax(tau, dmin);
  R base = dmin * inv_sc;
  base = base * base;
  R con = tau * inv_sc;
  R r0 = con * (dmin / d0), r1 = con * (dmin / d1), r2 = con * (dmin / d2);
  R w0 = base + r0 * r0, w1 = base + r1 * r1, w2 = base + r2 * r2;
  hi = wenoz_combine(m2, m1, c, p1, p2, w0, w1, w2);
  lo = wenoz_combine(p2, p1, c, m1, m2, w2, w1, w0);
}

template <int RECON, typename R>
__device__ __forceinline__ void edges(R m2, R m1, R c, R p1, R p2, R& lo, R& hi) {
  if constexpr (RECON == 0) edges_dc(m2, m1, c, p1, p2, lo, hi);
  else if constexpr (RECON == 1) edges_plm(m2, m1, c, p1, p2, lo, hi);
  else if constexpr (RECON == 2) edges_ppm4(m2, m1, c, p1, p2, lo, hi);
  else if constexpr (RECON == 3) edges_ppmx(m2, m1, c, p1, p2, lo, hi);
  else edges_wenoz(m2, m1, c, p1, p2, lo, hi);
}

// Ghost-cell depth a tile needs: the cells -1..n of a sweep use a stencil of
// half-width 0 (dc), 1 (plm) or 2 (ppm4/ppmx/wenoz); viscous gradients need 1.
template <int RECON> struct TileHalo { static constexpr int value = RECON == 0 ? 1 : (RECON == 1 ? 2 : 3); };

// ---------------------------------------------------------------------------
// Riemann solvers in the (normal, tangential) frame (fluxes.py:134-201).
// ---------------------------------------------------------------------------

template <typename R> struct Gas {
  R cs, cs2, inv_cs, half_inv_cs;
};

template <typename R>
__device__ __forceinline__ void flux_llf(R dl, R dr, R ul, R ur, R tl, R tr, const Gas<R>& g,
                                         R& f0, R& f1, R& f2) {
  // fluxes.py:175-183.
  R ml = dl * ul, mr = dr * ur;
  R ql = dl * tl, qr = dr * tr;
  R s0 = ml + mr;
  R s1 = ml * ul + mr * ur + g.cs2 * (dl + dr);
  R s2 = ml * tl + mr * tr;
  R sp = fmax(fabs(ul) + g.cs, fabs(ur) + g.cs);
  f0 = R(0.5) * (s0 - sp * (dr - dl));
  f1 = R(0.5) * (s1 - sp * (mr - ml));
  f2 = R(0.5) * (s2 - sp * (qr - ql));
}

template <typename R>
__device__ __forceinline__ void flux_hlle(R dl, R dr, R ul, R ur, R tl, R tr, const Gas<R>& g,
                                          R& f0, R& f1, R& f2) {
  // fluxes.py:186-201.
  R sl = sqrt(dl), sr = sqrt(dr);
  R u = (sl * ul + sr * ur) * (R(1) / (sl + sr));
  R alo = fmin(u - g.cs, ul - g.cs);
  R ahi = fmax(u + g.cs, ur + g.cs);
  R bm = alo < R(0) ? alo : R(-1e-20);
  R bp = ahi > R(0) ? ahi : R(1e-20);
  R vl = ul - bm, vr = ur - bp;
  R fl0 = dl * vl, fl1 = dl * ul * vl + g.cs2 * dl, fl2 = dl * tl * vl;
  R fr0 = dr * vr, fr1 = dr * ur * vr + g.cs2 * dr, fr2 = dr * tr * vr;
  R w = R(0.5) * (bp + bm) / (bp - bm);
  f0 = R(0.5) * (fl0 + fr0) + w * (fl0 - fr0);
  f1 = R(0.5) * (fl1 + fr1) + w * (fl1 - fr1);
  f2 = R(0.5) * (fl2 + fr2) + w * (fl2 - fr2);
}

template <typename R>
__device__ __forceinline__ void flux_roe(R dl, R dr, R ul, R ur, R tl, R tr, const Gas<R>& g,
                                         R& f0, R& f1, R& f2) {
  // fluxes.py:134-172.
  R ml = dl * ul, mr = dr * ur;
  R ql = dl * tl, qr = dr * tr;
  R pl = g.cs2 * dl, pr = g.cs2 * dr;
  R l0 = ml, l1 = ml * ul + pl, l2 = ml * tl;
  R r0 = mr, r1 = mr * ur + pr, r2 = mr * tr;
  R a0 = R(0.5) * (l0 + r0), a1 = R(0.5) * (l1 + r1), a2 = R(0.5) * (l2 + r2);
  R sl = sqrt(dl), sr = sqrt(dr);
  R inv = R(1) / (sl + sr);
  R u = (sl * ul + sr * ur) * inv;
  R t = (sl * tl + sr * tr) * inv;
  R lm = u - g.cs, lp = u + g.cs;
  R jd = dr - dl, jm = mr - ml, jq = qr - ql;
  R hu = (R(0.5) * u) * g.inv_cs;
  R jmc = jm * g.half_inv_cs;
  R am = jd * (R(0.5) + hu) - jmc;
  R az = jd * (-t) + jq;
  R ap = jd * (R(0.5) - hu) + jmc;
  R km = R(-0.5) * fabs(lm) * am;
  R kz = R(-0.5) * fabs(u) * az;
  R kp = R(-0.5) * fabs(lp) * ap;
  R g0 = a0 + km + kp;
  R g1 = a1 + km * lm + kp * lp;
  R g2 = a2 + km * t + kz + kp * t;
  if (lm >= R(0)) { g0 = l0; g1 = l1; g2 = l2; }
  if (lp <= R(0)) { g0 = r0; g1 = r1; g2 = r2; }
  R dstar = dl + am;
  if (dstar < R(0) || dstar + ap < R(0)) {
    R sp = R(0.5) * fmax(fabs(ul) + g.cs, fabs(ur) + g.cs);
    g0 = a0 - sp * jd;
    g1 = a1 - sp * jm;
    g2 = a2 - sp * jq;
  }
  f0 = g0;
  f1 = g1;
  f2 = g2;
}

template <int RS, typename R>
__device__ __forceinline__ void riemann(R dl, R dr, R ul, R ur, R tl, R tr, const Gas<R>& g,
                                        R& f0, R& f1, R& f2) {
  if constexpr (RS == 0) flux_llf(dl, dr, ul, ur, tl, tr, g, f0, f1, f2);
  else if constexpr (RS == 1) flux_hlle(dl, dr, ul, ur, tl, tr, g, f0, f1, f2);
  else flux_roe(dl, dr, ul, ur, tl, tr, g, f0, f1, f2);
}

// ---------------------------------------------------------------------------
// Reductions.
// ---------------------------------------------------------------------------

__device__ __forceinline__ double warp_nan_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ double warp_sum(double v) {
  // Fixed butterfly order: deterministic for a given lane assignment.
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide NaN-propagating max of K values; result valid in thread 0.
template <int K>
__device__ __forceinline__ void block_nan_max(double (&v)[K], double* scratch /* 32*K */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_nan_max(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) scratch[warp * K + k] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double x = lane < nwarp ? scratch[lane * K + k] : 0.0;
      v[k] = warp_nan_max(x);
    }
  }
}

// Block-wide sum of K values in a fixed order; result valid in thread 0.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* scratch /* 32*K */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) scratch[warp * K + k] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double x = lane < nwarp ? scratch[lane * K + k] : 0.0;
      v[k] = warp_sum(x);
    }
  }
}

__host__ __device__ __forceinline__ int wrap_index(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}

}  // namespace jx
