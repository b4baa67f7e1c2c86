// Device-side building blocks of the fused isothermal stage kernel: exact
// comparison/min/max primitives, the reconstructions split into a per-face
// and a per-cell part, Riemann solvers, and block reductions.
//
// Arithmetic follows the reference's operation order (jathenax/fluxes.py)
// with two deliberate changes that the float64 parity tolerance (1e-12
// relative per stage) covers: divisions by loop-invariant constants (12, 6,
// cs, dx, dy) become multiplications by the reciprocal, and nvcc contracts
// a*b+c into FMA.
//
// GB300 executes float64 at 2 FMA per SM per clock, 1/64 of float32, while
// the integer ALU is nearly idle in this kernel. For double precision the
// comparisons, sign tests, min/max and absolute-value tests therefore run on
// the IEEE bit patterns in the integer pipe. For every non-NaN operand they
// select exactly what the floating-point comparison selects (the only
// exception: a product a*b that underflows to +-0 is classified by the signs
// of a and b); NaN operands are treated as large numbers instead of being
// skipped by fmin/fmax, which only matters for a state that has already
// failed. Single precision uses the native instructions.
//
// Float32 arithmetic on the stage path has every rounding explicit
// (__fmul_rn / __fadd_rn / __fsub_rn / __fmaf_rn through Ops<float>, FMAs
// placed by hand): the compiler may not fuse a multiply into a neighbouring
// add on its own, because which pairs it would fuse depends on what else the
// thread computes (a product shared by two faces of one thread is not fused,
// the same product alone is). So every float32 kernel variant - shared-memory
// or register-marching tile, one to three columns per lane, lean or generic
// form, one solve or a batch - gives the same bits. Float64 keeps the plain
// operators and the compiler's contraction (its kernels' results are pinned
// by the parity tests, and its variants share one kernel family per use).
//
// Reciprocals and quotients (primitive recovery, Riemann solvers, PLM/PPMX/
// WENO-Z weights, CFL speeds) go through Num<R>::rcp/div. In float32 both use
// the special-function unit's approximations (PTX rcp.approx.f32,
// sqrt.approx.f32, about one unit in the last place). In float64 the
// reciprocals of the recovery, the Riemann solvers and the CFL speeds, and
// the square root of the Roe/HLLE average, are third-order refinements of
// the unit's float64 seeds (within an ulp; the tolerance against the
// reference is 1e-12 per stage), and the PLM, PPMX, WENO-Z and HLLE
// quotients multiply by such a reciprocal.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace jx {

template <typename R> struct Tiny;
template <> struct Tiny<double> { static constexpr double value = 2.2250738585072014e-308; };
template <> struct Tiny<float> { static constexpr float value = 1.17549435e-38f; };

// A compile-time boolean for dispatching a runtime flag once per kernel.
template <bool B> struct Flag { static constexpr bool value = B; };

// NaN-propagating max/min (jnp.maximum/minimum and the max/min reductions).
template <typename T> __device__ __forceinline__ T nan_max(T a, T b) {
  return (a > b || a != a) ? a : b;
}
template <typename T> __device__ __forceinline__ T nan_min(T a, T b) {
  return (a < b || a != a) ? a : b;
}

// ---------------------------------------------------------------------------
// Exact comparison primitives. Num<R>::f(...) has the semantics of the
// expression in its comment for non-NaN arguments.
// ---------------------------------------------------------------------------
template <typename R> struct Num;

template <> struct Num<float> {
  static __device__ __forceinline__ bool gt0(float x) { return x > 0.f; }          // x > 0
  static __device__ __forceinline__ bool lt0(float x) { return x < 0.f; }          // x < 0
  static __device__ __forceinline__ bool ge0(float x) { return x >= 0.f; }         // x >= 0
  static __device__ __forceinline__ bool le0(float x) { return x <= 0.f; }         // x <= 0
  static __device__ __forceinline__ float min(float a, float b) { return fminf(a, b); }
  static __device__ __forceinline__ float max(float a, float b) { return fmaxf(a, b); }
  // a, b >= 0 (no -0 ambiguity matters)
  static __device__ __forceinline__ float pmin(float a, float b) { return fminf(a, b); }
  static __device__ __forceinline__ float pmax(float a, float b) { return fmaxf(a, b); }
  static __device__ __forceinline__ bool pge(float a, float b) { return a >= b; }  // a, b >= 0
  static __device__ __forceinline__ bool pgt(float a, float b) { return a > b; }   // a, b >= 0
  static __device__ __forceinline__ bool prod_ge0(float a, float b) { return a * b >= 0.f; }
  static __device__ __forceinline__ bool prod_gt0(float a, float b) { return a * b > 0.f; }
  static __device__ __forceinline__ bool prod_le0(float a, float b) { return a * b <= 0.f; }
  // |a| >= 2|b|
  static __device__ __forceinline__ bool abs_ge_twice(float a, float b) { return fabsf(a) >= 2.f * fabsf(b); }
  static __device__ __forceinline__ bool lt(float a, float b) { return a < b; }    // a < b
  // max of a >= 0 and b >= 0 or NaN, propagating NaN
  static __device__ __forceinline__ float nanmax_pos(float a, float b) { return (b > a || b != b) ? b : a; }
  // 1/x, sqrt(x) and a/b from the special-function unit (see above)
  static __device__ __forceinline__ float rcp(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float root(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  // a/b as a (1/b), except where 1/b overflows (b zero or subnormal), b or a
  // is not finite: there a/b itself.
  static __device__ __forceinline__ float div(float a, float b) {
    const unsigned eb = (__float_as_uint(b) >> 23) & 0xff, ea = (__float_as_uint(a) >> 23) & 0xff;
    if (eb == 0 || eb == 0xff || ea == 0xff) return a / b;
    return __fmul_rn(a, rcp(b));
  }
  static __device__ __forceinline__ float quick_div(float a, float b) { return div(a, b); }
  // sqrt(a) sqrt(b) for a, b >= 0
  static __device__ __forceinline__ float geo_mean(float a, float b) { return __fmul_rn(root(a), root(b)); }
};

template <> struct Num<double> {
  static __device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
  static constexpr long long kSign = (long long)0x8000000000000000ULL;
  static constexpr long long kMag = 0x7fffffffffffffffLL;
  // Monotone integer key: a < b  <=>  key(a) < key(b); -0 sorts just below +0.
  static __device__ __forceinline__ long long key(double x) {
    long long b = bits(x);
    return b >= 0 ? b : (b ^ kMag);
  }
  static __device__ __forceinline__ bool zero(long long b) { return (b << 1) == 0; }
  static __device__ __forceinline__ bool gt0(double x) { return bits(x) > 0; }
  static __device__ __forceinline__ bool le0(double x) { return bits(x) <= 0; }
  static __device__ __forceinline__ bool lt0(double x) { long long b = bits(x); return b < 0 && b != kSign; }
  static __device__ __forceinline__ bool ge0(double x) { long long b = bits(x); return b >= 0 || b == kSign; }
  static __device__ __forceinline__ double min(double a, double b) { return key(a) <= key(b) ? a : b; }
  static __device__ __forceinline__ double max(double a, double b) { return key(a) >= key(b) ? a : b; }
  static __device__ __forceinline__ double pmin(double a, double b) { return bits(a) <= bits(b) ? a : b; }
  static __device__ __forceinline__ double pmax(double a, double b) { return bits(a) >= bits(b) ? a : b; }
  static __device__ __forceinline__ bool pge(double a, double b) { return bits(a) >= bits(b); }
  static __device__ __forceinline__ bool pgt(double a, double b) { return bits(a) > bits(b); }
  static __device__ __forceinline__ bool prod_ge0(double a, double b) {
    long long x = bits(a), y = bits(b);
    return (x ^ y) >= 0 || zero(x) || zero(y);
  }
  static __device__ __forceinline__ bool prod_gt0(double a, double b) {
    long long x = bits(a), y = bits(b);
    return (x ^ y) >= 0 && !zero(x) && !zero(y);
  }
  static __device__ __forceinline__ bool prod_le0(double a, double b) { return !prod_gt0(a, b); }
  static __device__ __forceinline__ bool abs_ge_twice(double a, double b) {
    // Doubling |b| adds one to the exponent field of a normal number and
    // doubles the bit pattern of a subnormal one.
    const long long ua = bits(a) & kMag, ub = bits(b) & kMag;
    const long long ub2 = ub < (1LL << 52) ? (ub << 1) : ub + (1LL << 52);
    return ua >= ub2;
  }
  static __device__ __forceinline__ bool lt(double a, double b) { return key(a) < key(b); }
  // max of a >= 0 and b >= 0 or NaN, propagating NaN (NaN of either sign
  // compares above +inf once the sign bit is cleared)
  static __device__ __forceinline__ double nanmax_pos(double a, double b) {
    const long long x = bits(a) & kMag, y = bits(b) & kMag;
    return y > x ? __longlong_as_double(y) : __longlong_as_double(x);
  }
  // True when x is zero, subnormal, below 2^-999, above 2^977, or not
  // finite: there the flush-to-zero seed below (or its reciprocal) leaves the
  // normal range, and the correctly rounded operation is used instead.
  static __device__ __forceinline__ bool outside_seed_range(double x) {
    const long long e = (bits(x) >> 52) & 0x7ff;  // biased exponent
    return e < 24 || e > 2000;
  }
  // 1/x refined from the special-function unit's seed y (PTX
  // rcp.approx.ftz.f64) by one third-order step of the series
  // 1/x = y / (1 - e) = y (1 + e + e^2 + ...), e = 1 - x y:
  // y <- y + y (e + e^2), which cubes the seed's relative error (Flynn, "On
  // division by functional iteration", IEEE TC 1970) — from the seed's
  // ~2^-23 to far below an ulp, leaving the final rounding: within an ulp of
  // 1/x (checked against correctly rounded division by the tests). Three
  // DFMA instead of the longer correctly rounded sequence; float64 parity
  // allows the ulp.
  static __device__ __forceinline__ double rcp(double x) {
    if (outside_seed_range(x)) return 1.0 / x;
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
  }
  static __device__ __forceinline__ double root(double x) { return sqrt(x); }
  // sqrt(a) sqrt(b) for a, b >= 0 with one square root, sqrt(a b), unless
  // the product leaves the normal range.
  static __device__ __forceinline__ double geo_mean(double a, double b) {
    const double p = a * b;
    const long long e = (bits(p) >> 52) & 0x7ff;
    if (e == 0 || e == 0x7ff) return sqrt(a) * sqrt(b);
    return outside_seed_range(p) ? sqrt(p) : sqrt_refined(p);
  }
  // sqrt(p) for p inside the seed range, from the special-function unit's
  // reciprocal square root y (PTX rsqrt.approx.ftz.f64): with t = p y and
  // e = 1 - t y = 1 - p y^2, sqrt(p) = t (1 - e)^(-1/2) = t (1 + e/2 + 3e^2/8
  // + ...); keeping two terms is one third-order step of the binomial series
  // (the Newton-Raphson family for x^(-1/2)), cubing the seed's ~2^-23
  // relative error. Five float64 operations; within an ulp of the correctly
  // rounded root (checked by the tests).
  static __device__ __forceinline__ double sqrt_refined(double p) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(p));
    const double t = p * y;
    const double e = fma(-t, y, 1.0);
    return fma(t, e * fma(e, 0.375, 0.5), t);
  }
  // a/b correctly rounded.
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  // a/b as a times the refined reciprocal of b (within about 1.5 ulp), the
  // product rounded on its own (__dmul_rn) so that no kernel can fuse it into
  // a neighbouring add. Used by the PLM, PPMX, WENO-Z and HLLE weights.
  static __device__ __forceinline__ double quick_div(double a, double b) {
    if (outside_seed_range(b)) return a / b;
    return __dmul_rn(a, rcp(b));
  }
};

// Explicitly rounded float32 operations (see the file comment); float64 maps
// to the plain operators, so an expression written with Ops<double> is the
// same expression the compiler saw before.
template <typename R> struct Ops;
template <> struct Ops<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
};
template <> struct Ops<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
};

// ---------------------------------------------------------------------------
// Reconstructions (fluxes.py:6-131). PPM4 and PPMX are split into the value
// at a face, which both neighbouring cells share, and a per-cell limiter
// that takes the cell's low/high face values; DC, PLM and WENO-Z produce the
// cell's low/high edges directly from its stencil.
// ---------------------------------------------------------------------------
template <int RECON> struct ReconTraits {
  static constexpr bool kFaceShared = RECON == 2 || RECON == 3;  // ppm4, ppmx
  static constexpr int kHalo = RECON == 0 ? 1 : (RECON == 1 ? 2 : 3);
};

// Products by 2 are written as explicit FMAs, a - 2b = fma(-2, b, a): the
// same single rounding (2b is exact), and the compiler would otherwise form
// 2b as b + b and lose the fusion, one more float64 operation each.

// Fourth-order interpolant at the face between w1 and w2 (fluxes.py:29-30).
template <typename R>
__device__ __forceinline__ R ppm_interp(R w0, R w1, R w2, R w3) {
  if constexpr (sizeof(R) == 4)
    return __fmul_rn(__fmaf_rn(7.f, __fadd_rn(w2, w1), -__fadd_rn(w0, w3)), float(1.0 / 12.0));
  return (R(7) * (w2 + w1) - (w0 + w3)) * R(1.0 / 12.0);
}

// PPM4 face value: interpolant bounded by the two neighbours (fluxes.py:29-32).
template <typename R>
__device__ __forceinline__ R ppm4_face(R w0, R w1, R w2, R w3) {
  using N = Num<R>;
  const R e = ppm_interp(w0, w1, w2, w3);
  return N::min(N::max(e, N::min(w2, w1)), N::max(w2, w1));
}

// PPM4 cell limiter (fluxes.py:35-42).
template <typename R>
__device__ __forceinline__ void ppm4_cell(R c, R lo_face, R hi_face, R& lo, R& hi) {
  using N = Num<R>;
  const R dh = hi_face - c;
  const R dl = lo_face - c;
  const bool flat = N::prod_ge0(dh, dl);
  const bool steep_lo = N::abs_ge_twice(dl, dh), steep_hi = N::abs_ge_twice(dh, dl);
  if constexpr (sizeof(R) == 8) {
    // The two steepening tests hold together only for dl = dh = 0, which is
    // flat: one FMA, on the selected difference, serves whichever applies
    // (one float64 operation fewer per variable and direction).
    const R x = fma(R(-2), steep_lo ? dh : dl, c);
    lo = flat ? c : (steep_lo ? x : lo_face);
    hi = flat ? c : (steep_hi ? x : hi_face);
  } else {
    const R l2 = steep_lo ? fma(R(-2), dh, c) : lo_face;
    const R h2 = steep_hi ? fma(R(-2), dl, c) : hi_face;
    lo = flat ? c : l2;
    hi = flat ? c : h2;
  }
}

// Smooth-extremum limiter of one face value (fluxes.py:45-53).
template <typename R>
__device__ __forceinline__ R ppmx_edge(R a, R b, R edge, R ca, R cb) {
  using N = Num<R>;
  using O = Ops<R>;
  const R curv = O::mul(R(3), fma(R(-2), edge, O::add(a, b)));
  const bool agree = (N::gt0(curv) && N::gt0(ca) && N::gt0(cb)) || (N::lt0(curv) && N::lt0(ca) && N::lt0(cb));
  const R mag = N::pmin(fabs(ca), fabs(cb));
  const R lim = copysign(N::pmin(O::mul(R(1.25), mag), fabs(curv)), curv);
  R fixed;
  if constexpr (sizeof(R) == 4) fixed = __fmaf_rn(-(agree ? lim : 0.f), float(1.0 / 6.0), __fmul_rn(0.5f, __fadd_rn(a, b)));
  else fixed = R(0.5) * (a + b) - (agree ? lim : R(0)) * R(1.0 / 6.0);
  return N::prod_gt0(O::sub(a, edge), O::sub(b, edge)) ? fixed : edge;
}

// PPMX face value between w1 and w2 (fluxes.py:62-68).
template <typename R>
__device__ __forceinline__ R ppmx_face(R w0, R w1, R w2, R w3) {
  const R e = ppm_interp(w0, w1, w2, w3);
  const R c1 = fma(R(-2), w1, w0 + w2);
  const R c2 = fma(R(-2), w2, w1 + w3);
  return ppmx_edge(w1, w2, e, c1, c2);
}

// PPMX cell limiter (fluxes.py:70-84).
template <typename R>
__device__ __forceinline__ void ppmx_cell(R m2, R m1, R c, R p1, R p2, R lo_face, R hi_face, R& lo, R& hi) {
  using N = Num<R>;
  const R cl = fma(R(-2), m1, m2 + c);
  const R cm = fma(R(-2), c, m1 + p1);
  const R cr = fma(R(-2), p1, c + p2);
  const R dh = hi_face - c;
  const R dl = lo_face - c;
  const bool ext = N::prod_le0(dh, c - lo_face) || N::prod_le0(m1 - c, c - p1);
  const R d2 = Ops<R>::mul(R(6), fma(R(-2), c, lo_face + hi_face));
  const bool agree = (N::gt0(d2) && N::gt0(cl) && N::gt0(cm) && N::gt0(cr)) ||
                     (N::lt0(d2) && N::lt0(cl) && N::lt0(cm) && N::lt0(cr));
  const R mag = N::pmin(fabs(cm), N::pmin(fabs(cl), fabs(cr)));
  const R lim = copysign(N::pmin(Ops<R>::mul(R(1.25), mag), fabs(d2)), d2);
  const R scale = N::pmax(fabs(m1), N::pmax(fabs(c), fabs(p1)));
  const bool use = agree && N::pgt(fabs(d2), Ops<R>::mul(R(1e-12), scale));
  R ratio = R(0);
  if (use) ratio = N::quick_div(lim, d2);
  const bool steep_lo = N::abs_ge_twice(dl, dh), steep_hi = N::abs_ge_twice(dh, dl);
  R lm, hm;
  if constexpr (sizeof(R) == 8) {
    // As in ppm4_cell: both tests hold only for dl = dh = 0, where both
    // results are c, so one FMA serves whichever applies.
    const R x = fma(R(-2), steep_lo ? dh : dl, c);
    lm = steep_lo ? x : lo_face;
    hm = steep_hi ? x : hi_face;
  } else {
    lm = steep_lo ? fma(R(-2), dh, c) : lo_face;
    hm = steep_hi ? fma(R(-2), dl, c) : hi_face;
  }
  if constexpr (sizeof(R) == 4) {
    lo = ext ? __fmaf_rn(dl, ratio, c) : lm;
    hi = ext ? __fmaf_rn(dh, ratio, c) : hm;
  } else {
    lo = ext ? c + dl * ratio : lm;
    hi = ext ? c + dh * ratio : hm;
  }
}

template <typename R>
__device__ __forceinline__ void plm_cell(R m1, R c, R p1, R& lo, R& hi) {
  // fluxes.py:11-18, harmonic-mean slope.
  using N = Num<R>;
  const R bw = c - m1;
  const R fw = p1 - c;
  using O = Ops<R>;
  R hs = R(0);
  if (N::prod_gt0(bw, fw)) hs = N::quick_div(O::mul(bw, fw), O::add(bw, fw));
  hi = O::add(c, hs);
  lo = O::sub(c, hs);
}

// Float64 WENO-Z with every rounding spelled out (explicit FMAs and
// unfusable _rn operations): the compiler has no contraction left to choose,
// so every kernel instantiation forms the same bits, and the quotients can
// use the refined reciprocal (quick_div) without the batched and
// single-solve kernels drifting apart in the last bit.
__device__ __forceinline__ double wenoz_combine_f64(double s0, double s1, double s2, double s3, double s4,
                                                     double w0, double w1, double w2) {
  // fluxes.py:87-93.
  const double a0 = __dmul_rn(0.1, w0), a1 = __dmul_rn(0.6, w1), a2 = __dmul_rn(0.3, w2);
  const double f0 = fma(11.0, s2, fma(-7.0, s1, __dmul_rn(2.0, s0)));
  const double f1 = fma(2.0, s3, fma(5.0, s2, -s1));
  const double f2 = __dsub_rn(fma(5.0, s3, __dmul_rn(2.0, s2)), s4);
  const double num = fma(f2, a2, fma(f1, a1, __dmul_rn(f0, a0)));
  const double den = __dmul_rn(6.0, __dadd_rn(__dadd_rn(a0, a1), a2));
  return Num<double>::quick_div(num, den);
}

__device__ __forceinline__ void wenoz_cell_f64(double m2, double m1, double c, double p1, double p2, double& lo,
                                               double& hi) {
  // fluxes.py:96-117; eps = max(1e-42, finfo(float64).tiny) at fluxes.py:108.
  using N = Num<double>;
  const double k1312 = 13.0 / 12.0, eps = 1e-42;
  const double t0 = fma(-2.0, m1, __dadd_rn(m2, c)), u0 = fma(-4.0, m1, fma(3.0, c, m2));
  const double t1 = fma(-2.0, c, __dadd_rn(m1, p1)), u1 = __dsub_rn(m1, p1);
  const double t2 = fma(-2.0, p1, __dadd_rn(p2, c)), u2 = fma(-4.0, p1, fma(3.0, c, p2));
  const double b0 = fma(k1312, __dmul_rn(t0, t0), __dmul_rn(0.25, __dmul_rn(u0, u0)));
  const double b1 = fma(k1312, __dmul_rn(t1, t1), __dmul_rn(0.25, __dmul_rn(u1, u1)));
  const double b2 = fma(k1312, __dmul_rn(t2, t2), __dmul_rn(0.25, __dmul_rn(u2, u2)));
  const double tau = fabs(__dsub_rn(b0, b2));
  const double d0 = __dadd_rn(b0, eps), d1 = __dadd_rn(b1, eps), d2 = __dadd_rn(b2, eps);
  const double dmin = N::pmin(d0, N::pmin(d1, d2));
  const double inv_sc = N::quick_div(1.0, N::pmax(tau, dmin));
  double base = __dmul_rn(dmin, inv_sc);
  base = __dmul_rn(base, base);
  const double con = __dmul_rn(tau, inv_sc);
  const double r0 = __dmul_rn(con, N::quick_div(dmin, d0));
  const double r1 = __dmul_rn(con, N::quick_div(dmin, d1));
  const double r2 = __dmul_rn(con, N::quick_div(dmin, d2));
  const double w0 = fma(r0, r0, base), w1 = fma(r1, r1, base), w2 = fma(r2, r2, base);
  hi = wenoz_combine_f64(m2, m1, c, p1, p2, w0, w1, w2);
  lo = wenoz_combine_f64(p2, p1, c, m1, m2, w2, w1, w0);
}

// Float32 (float64 uses wenoz_combine_f64): every rounding explicit.
__device__ __forceinline__ float wenoz_combine(float s0, float s1, float s2, float s3, float s4, float w0, float w1,
                                               float w2) {
  // fluxes.py:87-93.
  const float a0 = __fmul_rn(0.1f, w0), a1 = __fmul_rn(0.6f, w1), a2 = __fmul_rn(0.3f, w2);
  const float f0 = __fmaf_rn(11.f, s2, __fmaf_rn(-7.f, s1, __fmul_rn(2.f, s0)));
  const float f1 = __fmaf_rn(2.f, s3, __fmaf_rn(5.f, s2, -s1));
  const float f2 = __fsub_rn(__fmaf_rn(5.f, s3, __fmul_rn(2.f, s2)), s4);
  const float num = __fmaf_rn(f2, a2, __fmaf_rn(f1, a1, __fmul_rn(f0, a0)));
  return Num<float>::div(num, __fmul_rn(6.f, __fadd_rn(__fadd_rn(a0, a1), a2)));
}

__device__ __forceinline__ void wenoz_cell_f32(float m2, float m1, float c, float p1, float p2, float& lo,
                                               float& hi) {
  // fluxes.py:96-117; eps = max(1e-42, finfo(float32).tiny) at fluxes.py:108.
  using N = Num<float>;
  const float k1312 = float(13.0 / 12.0);
  const float eps = 1e-42f > Tiny<float>::value ? 1e-42f : Tiny<float>::value;
  const float t0 = __fmaf_rn(-2.f, m1, __fadd_rn(m2, c)), u0 = __fmaf_rn(-4.f, m1, __fmaf_rn(3.f, c, m2));
  const float t1 = __fmaf_rn(-2.f, c, __fadd_rn(m1, p1)), u1 = __fsub_rn(m1, p1);
  const float t2 = __fmaf_rn(-2.f, p1, __fadd_rn(p2, c)), u2 = __fmaf_rn(-4.f, p1, __fmaf_rn(3.f, c, p2));
  const float b0 = __fmaf_rn(k1312, __fmul_rn(t0, t0), __fmul_rn(0.25f, __fmul_rn(u0, u0)));
  const float b1 = __fmaf_rn(k1312, __fmul_rn(t1, t1), __fmul_rn(0.25f, __fmul_rn(u1, u1)));
  const float b2 = __fmaf_rn(k1312, __fmul_rn(t2, t2), __fmul_rn(0.25f, __fmul_rn(u2, u2)));
  const float tau = fabsf(__fsub_rn(b0, b2));
  const float d0 = __fadd_rn(b0, eps), d1 = __fadd_rn(b1, eps), d2 = __fadd_rn(b2, eps);
  const float dmin = N::pmin(d0, N::pmin(d1, d2));
  const float inv_sc = N::div(1.f, N::pmax(tau, dmin));
  float base = __fmul_rn(dmin, inv_sc);
  base = __fmul_rn(base, base);
  const float con = __fmul_rn(tau, inv_sc);
  const float r0 = __fmul_rn(con, N::div(dmin, d0)), r1 = __fmul_rn(con, N::div(dmin, d1)),
              r2 = __fmul_rn(con, N::div(dmin, d2));
  const float w0 = __fmaf_rn(r0, r0, base), w1 = __fmaf_rn(r1, r1, base), w2 = __fmaf_rn(r2, r2, base);
  hi = wenoz_combine(m2, m1, c, p1, p2, w0, w1, w2);
  lo = wenoz_combine(p2, p1, c, m1, m2, w2, w1, w0);
}

template <typename R>
__device__ __forceinline__ void wenoz_cell(R m2, R m1, R c, R p1, R p2, R& lo, R& hi) {
  if constexpr (sizeof(R) == 8) wenoz_cell_f64(m2, m1, c, p1, p2, lo, hi);
  else wenoz_cell_f32(m2, m1, c, p1, p2, lo, hi);
}

// RK4's saved register (hydro.py:46-50 with delta): V + delta U.
template <typename R>
__device__ __forceinline__ R delta_update(R v, R delta, R u) {
  if constexpr (sizeof(R) == 4) return __fmaf_rn(delta, u, v);
  else return v + delta * u;
}

// RK stage combine of one component (hydro.py:39-51): the blend form
// V + g0 (U - V) - beta dt div, else g0 U + g1 V - beta dt div, with
// div = dFx/dx + dFy/dy. The flux differences enter through fused
// multiply-adds with ncx = -beta dt/dx and ncy = -beta dt/dy (per launch),
// which saves two float64 operations per component against forming div first.
// Zero flux differences leave the blend form exact (U = V gives V).
template <typename R>
__device__ __forceinline__ R rk_combine(bool blend, R g0, R g1, R u, R v, R dfx, R dfy, R ncx, R ncy) {
  const R base = blend ? fma(g0, u - v, v) : fma(g0, u, g1 * v);
  return fma(ncy, dfy, fma(ncx, dfx, base));
}

// Face value shared by the two cells at a face (PPM4/PPMX only).
template <int RECON, typename R>
__device__ __forceinline__ R face_value(R w0, R w1, R w2, R w3) {
  if constexpr (RECON == 2) return ppm4_face(w0, w1, w2, w3);
  else return ppmx_face(w0, w1, w2, w3);
}

// Low/high edges of the cell at the centre of (m2, m1, c, p1, p2); for the
// face-shared methods lo_face/hi_face are the cell's two face values.
template <int RECON, typename R>
__device__ __forceinline__ void cell_edges(R m2, R m1, R c, R p1, R p2, R lo_face, R hi_face,
                                           R& lo, R& hi) {
  if constexpr (RECON == 0) { lo = c; hi = c; }
  else if constexpr (RECON == 1) plm_cell(m1, c, p1, lo, hi);
  else if constexpr (RECON == 2) ppm4_cell(c, lo_face, hi_face, lo, hi);
  else if constexpr (RECON == 3) ppmx_cell(m2, m1, c, p1, p2, lo_face, hi_face, lo, hi);
  else wenoz_cell(m2, m1, c, p1, p2, lo, hi);
}

// Both edges of a cell from its 5-point stencil (+1 more on each side for
// the face-shared methods): used by the standalone face-state kernel.
template <int RECON, typename R>
__device__ __forceinline__ void edges_from_stencil(R m3, R m2, R m1, R c, R p1, R p2, R p3, R& lo, R& hi) {
  R lf = R(0), hf = R(0);
  if constexpr (ReconTraits<RECON>::kFaceShared) {
    lf = face_value<RECON>(m2, m1, c, p1);
    hf = face_value<RECON>(m1, c, p1, p2);
  }
  (void)m3;
  (void)p3;
  cell_edges<RECON>(m2, m1, c, p1, p2, lf, hf, lo, hi);
}

// ---------------------------------------------------------------------------
// Riemann solvers in the (normal, tangential) frame (fluxes.py:134-201).
// ---------------------------------------------------------------------------
template <typename R> struct Gas {
  R cs, cs2, inv_cs, half_inv_cs, quarter_inv_cs;
};

template <typename R>
__device__ __forceinline__ void flux_llf(R dl, R dr, R ul, R ur, R tl, R tr, const Gas<R>& g,
                                         R& f0, R& f1, R& f2) {
  // fluxes.py:175-183.
  using N = Num<R>;
  if constexpr (sizeof(R) == 4) {
    const float ml = __fmul_rn(dl, ul), mr = __fmul_rn(dr, ur);
    const float ql = __fmul_rn(dl, tl), qr = __fmul_rn(dr, tr);
    const float s0 = __fadd_rn(ml, mr);
    const float s1 = __fmaf_rn(ml, ul, __fmaf_rn(mr, ur, __fmul_rn(g.cs2, __fadd_rn(dl, dr))));
    const float s2 = __fmaf_rn(ml, tl, __fmul_rn(mr, tr));
    const float sp = N::pmax(__fadd_rn(fabsf(ul), g.cs), __fadd_rn(fabsf(ur), g.cs));
    f0 = __fmul_rn(0.5f, __fmaf_rn(-sp, __fsub_rn(dr, dl), s0));
    f1 = __fmul_rn(0.5f, __fmaf_rn(-sp, __fsub_rn(mr, ml), s1));
    f2 = __fmul_rn(0.5f, __fmaf_rn(-sp, __fsub_rn(qr, ql), s2));
    return;
  }
  const R ml = dl * ul, mr = dr * ur;
  const R ql = dl * tl, qr = dr * tr;
  const R s0 = ml + mr;
  const R s1 = ml * ul + mr * ur + g.cs2 * (dl + dr);
  const R s2 = ml * tl + mr * tr;
  const R sp = N::pmax(fabs(ul) + g.cs, fabs(ur) + g.cs);
  f0 = R(0.5) * (s0 - sp * (dr - dl));
  f1 = R(0.5) * (s1 - sp * (mr - ml));
  f2 = R(0.5) * (s2 - sp * (qr - ql));
}

template <typename R>
__device__ __forceinline__ void flux_hlle(R dl, R dr, R ul, R ur, R tl, R tr, const Gas<R>& g,
                                          R& f0, R& f1, R& f2) {
  // fluxes.py:186-201.
  using N = Num<R>;
  // Roe average (sl ul + sr ur) / (sl + sr), sl = sqrt(dl), sr = sqrt(dr),
  // multiplied through by sl: (dl ul + r ur) / (dl + r), r = sqrt(dl dr).
  if constexpr (sizeof(R) == 4) {
    const float r = N::geo_mean(dl, dr);
    const float u = __fmul_rn(__fmaf_rn(r, ur, __fmul_rn(dl, ul)), N::rcp(__fadd_rn(dl, r)));
    const float alo = N::min(__fsub_rn(u, g.cs), __fsub_rn(ul, g.cs));
    const float ahi = N::max(__fadd_rn(u, g.cs), __fadd_rn(ur, g.cs));
    const float bm = N::lt0(alo) ? alo : -1e-20f;
    const float bp = N::gt0(ahi) ? ahi : 1e-20f;
    const float vl = __fsub_rn(ul, bm), vr = __fsub_rn(ur, bp);
    const float ml = __fmul_rn(dl, ul), mr = __fmul_rn(dr, ur);
    const float fl0 = __fmul_rn(dl, vl), fl1 = __fmaf_rn(ml, vl, __fmul_rn(g.cs2, dl)), fl2 = __fmul_rn(__fmul_rn(dl, tl), vl);
    const float fr0 = __fmul_rn(dr, vr), fr1 = __fmaf_rn(mr, vr, __fmul_rn(g.cs2, dr)), fr2 = __fmul_rn(__fmul_rn(dr, tr), vr);
    const float w = N::quick_div(__fmul_rn(0.5f, __fadd_rn(bp, bm)), __fsub_rn(bp, bm));
    f0 = __fmaf_rn(w, __fsub_rn(fl0, fr0), __fmul_rn(0.5f, __fadd_rn(fl0, fr0)));
    f1 = __fmaf_rn(w, __fsub_rn(fl1, fr1), __fmul_rn(0.5f, __fadd_rn(fl1, fr1)));
    f2 = __fmaf_rn(w, __fsub_rn(fl2, fr2), __fmul_rn(0.5f, __fadd_rn(fl2, fr2)));
    return;
  }
  const R r = N::geo_mean(dl, dr);
  const R u = fma(r, ur, dl * ul) * N::rcp(dl + r);
  const R alo = N::min(u - g.cs, ul - g.cs);
  const R ahi = N::max(u + g.cs, ur + g.cs);
  const R bm = N::lt0(alo) ? alo : R(-1e-20);
  const R bp = N::gt0(ahi) ? ahi : R(1e-20);
  const R vl = ul - bm, vr = ur - bp;
  const R fl0 = dl * vl, fl1 = dl * ul * vl + g.cs2 * dl, fl2 = dl * tl * vl;
  const R fr0 = dr * vr, fr1 = dr * ur * vr + g.cs2 * dr, fr2 = dr * tr * vr;
  const R w = N::quick_div(R(0.5) * (bp + bm), bp - bm);
  f0 = R(0.5) * (fl0 + fr0) + w * (fl0 - fr0);
  f1 = R(0.5) * (fl1 + fr1) + w * (fl1 - fr1);
  f2 = R(0.5) * (fl2 + fr2) + w * (fl2 - fr2);
}

// Float32 Roe flux (fluxes.py:134-172), every rounding explicit. The Roe
// average makes A (U_r - U_l) = F_r - F_l exactly, so with all three wave
// speeds of one sign the dissipation formula already equals the upwind flux
// F_l or F_r (fluxes.py:165-166); float32, held to the float64 result only to
// rounding, relies on that and skips the two selects (four ALU instructions
// per face in the issue-bound float32 kernels).
__device__ __forceinline__ void flux_roe_f32(float dl, float dr, float ul, float ur, float tl, float tr,
                                             const Gas<float>& g, float& f0, float& f1, float& f2) {
  using N = Num<float>;
  const float ml = __fmul_rn(dl, ul), mr = __fmul_rn(dr, ur);
  const float ql = __fmul_rn(dl, tl), qr = __fmul_rn(dr, tr);
  const float s0 = __fadd_rn(ml, mr);
  const float s1 = __fmaf_rn(ml, ul, __fmaf_rn(mr, ur, __fmul_rn(g.cs2, __fadd_rn(dl, dr))));
  const float s2 = __fmaf_rn(ml, tl, __fmul_rn(mr, tr));
  const float r = N::geo_mean(dl, dr);
  const float inv = N::rcp(__fadd_rn(dl, r));
  const float u = __fmul_rn(__fmaf_rn(r, ur, ml), inv);
  const float t = __fmul_rn(__fmaf_rn(r, tr, ql), inv);
  const float lm = __fsub_rn(u, g.cs), lp = __fadd_rn(u, g.cs);
  const float jd = __fsub_rn(dr, dl), jm = __fsub_rn(mr, ml), jq = __fsub_rn(qr, ql);
  // Wave strengths am = jd (1/2 + u/(2cs)) - jm/(2cs), az = jq - jd t,
  // ap = jd (1/2 - u/(2cs)) + jm/(2cs) (fluxes.py:150-153).
  const float hu = __fmul_rn(u, g.half_inv_cs);
  const float jmc = __fmul_rn(jm, g.half_inv_cs);
  const float am = __fmaf_rn(jd, __fadd_rn(0.5f, hu), -jmc);
  const float ap = __fmaf_rn(jd, __fsub_rn(0.5f, hu), jmc);
  const float az = __fmaf_rn(jd, -t, jq);
  const float wm = __fmul_rn(fabsf(lm), am), wz = __fmul_rn(fabsf(u), az), wp = __fmul_rn(fabsf(lp), ap);
  const float wmp = __fadd_rn(wm, wp);
  const float dstar = __fadd_rn(dl, am);
  const float dstar2 = __fadd_rn(dstar, ap);
  if (__builtin_expect(N::lt0(dstar) || N::lt0(dstar2), 0)) {  // positivity fix: rare
    const float sp = __fmul_rn(0.5f, N::pmax(__fadd_rn(fabsf(ul), g.cs), __fadd_rn(fabsf(ur), g.cs)));
    f0 = __fmaf_rn(-sp, jd, __fmul_rn(0.5f, s0));
    f1 = __fmaf_rn(-sp, jm, __fmul_rn(0.5f, s1));
    f2 = __fmaf_rn(-sp, jq, __fmul_rn(0.5f, s2));
    return;
  }
  f0 = __fmul_rn(0.5f, __fsub_rn(s0, wmp));
  f1 = __fmul_rn(0.5f, __fsub_rn(s1, __fmaf_rn(wm, lm, __fmul_rn(wp, lp))));
  f2 = __fmul_rn(0.5f, __fsub_rn(s2, __fmaf_rn(wmp, t, wz)));
}

template <typename R>
__device__ __forceinline__ void flux_roe(R dl, R dr, R ul, R ur, R tl, R tr, const Gas<R>& g,
                                         R& f0, R& f1, R& f2) {
  // fluxes.py:134-172.
  if constexpr (sizeof(R) == 4) {
    flux_roe_f32(dl, dr, ul, ur, tl, tr, g, f0, f1, f2);
  } else {
    using N = Num<R>;
    const R ml = dl * ul, mr = dr * ur;
    const R ql = dl * tl, qr = dr * tr;
    const R l0 = ml, l1 = ml * ul + g.cs2 * dl, l2 = ml * tl;
    const R r0 = mr, r1 = mr * ur + g.cs2 * dr, r2 = mr * tr;
    // Roe averages (sl v_l + sr v_r) / (sl + sr), sl = sqrt(dl), sr = sqrt(dr),
    // multiplied through by sl: (dl v_l + r v_r) / (dl + r), r = sqrt(dl dr).
    const R r = N::geo_mean(dl, dr);
    const R inv = N::rcp(dl + r);
    const R u = fma(r, ur, ml) * inv;
    const R t = fma(r, tr, ql) * inv;
    const R lm = u - g.cs, lp = u + g.cs;
    const R jd = dr - dl, jm = mr - ml, jq = qr - ql;
    // Wave strengths am = jd (1/2 + u/(2cs)) - jm/(2cs), az = jq - jd t,
    // ap = jd (1/2 - u/(2cs)) + jm/(2cs) (fluxes.py:150-153);
    // g = (l + r)/2 - (|lm| am e_m + |u| az e_z + |lp| ap e_p)/2 with the
    // eigenvectors e_m = (1, lm, t), e_z = (0, 0, 1), e_p = (1, lp, t).
    // am, ap and |u| az are formed halved and each component of g is one FMA
    // (two float64 operations fewer per face); am = jd/2 + X/(2cs),
    // ap = jd/2 - X/(2cs) with X = u jd - jm: one FMA for X serves both (two
    // float64 operations fewer per face).
    const R s0 = l0 + r0, s1 = l1 + r1, s2 = l2 + r2;
    const R az = fma(jd, -t, jq);
    const R X = fma(u, jd, -jm);
    const R jq4 = R(0.25) * jd;
    const R am = fma(X, g.quarter_inv_cs, jq4);   // am / 2
    const R ap = fma(-X, g.quarter_inv_cs, jq4);  // ap / 2
    const R wm = fabs(lm) * am, wz = (R(0.5) * fabs(u)) * az, wp = fabs(lp) * ap;  // halves
    const R wmp = wm + wp;
    R g0 = fma(R(0.5), s0, -wmp);
    R g1 = fma(R(0.5), s1, -fma(wm, lm, wp * lp));
    R g2 = fma(R(0.5), s2, -fma(wmp, t, wz));
    const R dstar = fma(R(2), am, dl);  // dl + am
    const R dstar2 = fma(R(2), ap, dstar);
    // Supersonic faces take the upwind flux (fluxes.py:165-166).
    if (N::ge0(lm)) { g0 = l0; g1 = l1; g2 = l2; }
    if (N::le0(lp)) { g0 = r0; g1 = r1; g2 = r2; }
    if (__builtin_expect(N::lt0(dstar) || N::lt0(dstar2), 0)) {  // positivity fix: rare
      const R sp = R(0.5) * N::pmax(fabs(ul) + g.cs, fabs(ur) + g.cs);
      g0 = R(0.5) * s0 - sp * jd;
      g1 = R(0.5) * s1 - sp * jm;
      g2 = R(0.5) * s2 - sp * jq;
    }
    f0 = g0;
    f1 = g1;
    f2 = g2;
  }
}

// Viscous momentum flux at a face (fluxes.py:227-266), added to (f1, f2):
// DIR 0 an x face, DIR 1 a y face, between cell a (low side) and cell b
// (high side) with velocities (ax, ay), (bx, by) and densities rho_a,
// rho_b; (tpx, tpy) and (tmx, tmy) are the transverse sums (b+ + a+) and
// (b- + a-) of the velocity one cell beyond the face on either side.
// inv_dn = 1/dx (x face) or 1/dy, inv_4dt = 1/(4 dy) or 1/(4 dx); nu the
// uniform viscosity, smag_c = Cs^2 dx dy (Smagorinsky when smag).
template <int DIR, typename R>
__device__ __forceinline__ void viscous_face(bool smag, R nu0, R smag_c, R inv_dn, R inv_4dt, R rho_a, R rho_b,
                                             R ax, R ay, R bx, R by, R tpx, R tpy, R tmx, R tmy, R& f1, R& f2) {
  if constexpr (sizeof(R) == 4) {
    const float dn_x = __fmul_rn(__fsub_rn(bx, ax), inv_dn), dn_y = __fmul_rn(__fsub_rn(by, ay), inv_dn);
    const float dt_x = __fmul_rn(__fsub_rn(tpx, tmx), inv_4dt), dt_y = __fmul_rn(__fsub_rn(tpy, tmy), inv_4dt);
    const float dvx_dx = DIR == 0 ? dn_x : dt_x, dvy_dx = DIR == 0 ? dn_y : dt_y;
    const float dvx_dy = DIR == 0 ? dt_x : dn_x, dvy_dy = DIR == 0 ? dt_y : dn_y;
    const float shear = __fadd_rn(dvy_dx, dvx_dy);
    const float s0 = DIR == 0 ? __fmaf_rn(float(4.0 / 3.0), dvx_dx, -__fmul_rn(float(2.0 / 3.0), dvy_dy)) : shear;
    const float s1 = DIR == 0 ? shear : __fmaf_rn(float(4.0 / 3.0), dvy_dy, -__fmul_rn(float(2.0 / 3.0), dvx_dx));
    float nu = nu0;
    if (smag) {
      const float s2 = __fmaf_rn(shear, shear, __fmul_rn(2.f, __fmaf_rn(dvx_dx, dvx_dx, __fmul_rn(dvy_dy, dvy_dy))));
      nu = __fmaf_rn(smag_c, sqrtf(s2), nu);
    }
    const float mu = __fmul_rn(__fmul_rn(0.5f, nu), __fadd_rn(rho_b, rho_a));
    f1 = __fmaf_rn(-mu, s0, f1);
    f2 = __fmaf_rn(-mu, s1, f2);
  } else {
    R dvx_dx, dvy_dx, dvx_dy, dvy_dy;
    if (DIR == 0) {
      dvx_dx = (bx - ax) * inv_dn;
      dvy_dx = (by - ay) * inv_dn;
      dvx_dy = (tpx - tmx) * inv_4dt;
      dvy_dy = (tpy - tmy) * inv_4dt;
    } else {
      dvx_dy = (bx - ax) * inv_dn;
      dvy_dy = (by - ay) * inv_dn;
      dvx_dx = (tpx - tmx) * inv_4dt;
      dvy_dx = (tpy - tmy) * inv_4dt;
    }
    const R shear = dvy_dx + dvx_dy;
    R s0, s1;
    if (DIR == 0) {
      s0 = R(4.0 / 3.0) * dvx_dx - R(2.0 / 3.0) * dvy_dy;
      s1 = shear;
    } else {
      s0 = shear;
      s1 = R(4.0 / 3.0) * dvy_dy - R(2.0 / 3.0) * dvx_dx;
    }
    R nu = nu0;
    if (smag) {
      const R s2 = R(2) * (dvx_dx * dvx_dx + dvy_dy * dvy_dy) + shear * shear;
      nu = nu + smag_c * sqrt(s2);
    }
    const R mu = (R(0.5) * nu) * (rho_b + rho_a);
    f1 = f1 + -(mu * s0);
    f2 = f2 + -(mu * s1);
  }
}

// Half the sum of two face-adjacent SGS stress values added to a flux
// component (fluxes.py:269-280).
template <typename R>
__device__ __forceinline__ R add_half_sum(R f, R ta, R tb) {
  if constexpr (sizeof(R) == 4) return __fmaf_rn(0.5f, __fadd_rn(ta, tb), f);
  else return f + R(0.5) * (ta + tb);
}

// Passive-scalar flux: the mass flux times the upwind concentration
// (fluxes.py:215-218).
template <typename R>
__device__ __forceinline__ R scalar_flux(R f0, R left, R right) {
  return Ops<R>::mul(f0, Num<R>::ge0(f0) ? left : right);
}

// Linear drag on one momentum component with the incoming density and
// velocity (hydro.py:122-125): m - (beta dt rate rho) v.
template <typename R>
__device__ __forceinline__ R drag_term(R m, R kdrag_rho, R v) {
  if constexpr (sizeof(R) == 4) return __fmaf_rn(-kdrag_rho, v, m);
  else return m + -(kdrag_rho * v);
}

// CFL signal speed |m / rho| + cs with inv = 1/rho.
template <typename R>
__device__ __forceinline__ R signal_speed(R inv, R m, R cs) {
  return Ops<R>::add(fabs(Ops<R>::mul(inv, m)), cs);
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
// Max reductions are exact, so reducing in float32 and widening the result
// gives the same float64 value as widening every input first.
template <typename T>
__device__ __forceinline__ T warp_nan_max(T v) {
  for (int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ double warp_sum(double v) {
  // Fixed butterfly order: deterministic for a given lane assignment.
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide NaN-propagating max of K values; result valid in thread 0.
template <int K, typename T>
__device__ __forceinline__ void block_nan_max(T (&v)[K], T* scratch /* 32*K */) {
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
      T x = lane < nwarp ? scratch[lane * K + k] : T(0);
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
