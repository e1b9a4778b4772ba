// Table-driven FP64 exp / log / pow for the FP64-pipe-bound NSW6 kernels.
//
// On GB300 the FP64 pipe issues about 2 operations per SM per cycle, so the
// number of FP64 instructions per transcendental decides the speed of the
// microphysics.  These routines follow the table-driven method of
// P. T. P. Tang ("Table-driven implementation of the exponential function in
// IEEE floating-point arithmetic", ACM TOMS 15(2), 1989; "Table-driven
// implementation of the logarithm function ...", ACM TOMS 16(4), 1990):
//
//   exp(x) = 2^m * 2^(j/256) * exp(r),  x = (256 m + j) ln2/256 + r,
//            |r| <= ln2/512, exp(r) - 1 by its degree-4 Taylor polynomial
//            (truncation error < 4e-17), 2^(j/256) = T_j (1 + d_j) from two
//            256-entry tables (T_j rounded, d_j its relative rounding error);
//   log(x) = e ln2 + log(c_j) + log1p(r),  x = 2^e m, m in [0.75, 1.5),
//            r = m / c_j - 1 with |r| < 2e-3, log1p(r) by its degree-6
//            Taylor polynomial, 1/c_j and -log(1/c_j) from 256-entry tables.
//
// Both are accurate to about half a unit in the last place; arguments outside
// the fast range (non-normal, huge, negative log arguments) fall back to the
// CUDA math library.  pow(x, y) = exp(y log x) carries the rounding error of
// y*log(x) (computed with a fused multiply-add) into exp through exp(h + l) =
// exp(h)(1 + l), which keeps it within a few units in the last place.
//
// The tables (8 KB) are built on the host in extended precision and staged
// in shared memory by every CTA.  The range tests compare bit patterns on the
// integer pipe (nsw6_fpcmp.cuh), with the IEEE comparisons' results.
#pragma once

#include <cstdint>

#include "nsw6_fpcmp.cuh"

namespace nsw6 {

constexpr int FM_EXP_N = 256;
constexpr int FM_LOG_N = 256;
constexpr int FM_TABLE_DOUBLES = 2 * FM_EXP_N + 2 * FM_LOG_N;

struct FastMath {
  const double* exp_t;    // [256]: 2^(j/256) rounded
  const double* exp_d;    // [256]: 2^(j/256) / exp_t[j] - 1
  const double* log_ic;   // [256]: 1 / c_j (rounded)
  const double* log_c;    // [256]: -log(log_ic[j])

  // exp within about half an ulp; slow path outside (-708, 708).
  __device__ __forceinline__ double exp(double x) const {
    if (!fp_abs_lt(x, 708.0)) return ::exp(x);
    const double shift = 6755399441055744.0;               // 1.5 * 2^52
    const double inv = 369.32993046757463;                  // 256 / ln 2
    const double l_hi = 2.7076061740622863e-03;             // ln2/256, high part
    const double l_lo = 9.058776616587108e-20;              // ln2/256 - l_hi
    const double t = __fma_rn(x, inv, shift);
    const double kd = __dadd_rn(t, -shift);
    double r = __fma_rn(kd, -l_hi, x);
    r = __fma_rn(kd, -l_lo, r);
    const int k = (int)__double2loint(t);
    const int j = k & (FM_EXP_N - 1);
    const int m = k >> 8;
    // exp(r) - 1 = r + r^2/2 + r^3/6 + r^4/24
    double p = __fma_rn(r, 4.1666666666666664e-02, 1.6666666666666666e-01);
    p = __fma_rn(p, r, 0.5);
    p = __fma_rn(p, r, 1.0);
    p = __fma_rn(p, r, exp_d[j]);   // exp(r) (1 + d_j) - 1, dropping d_j (exp(r) - 1) < 2e-19
    const long long tb = __double_as_longlong(exp_t[j]) + ((long long)m << 52);
    const double s = __longlong_as_double(tb);
    return __fma_rn(s, p, s);
  }

  // log(x) as hi + lo (|lo| <= ulp(hi)); slow path for x <= 0, non-normal, inf, nan.
  __device__ __forceinline__ double log_hl(double x, double& lo) const {
    const long long bits = __double_as_longlong(x);
    // x normal and finite, positive (the signed bits order the positive doubles)
    if (!(bits >= 0x0010000000000000ll && bits < 0x7FEFFFFFFFFFFFFFll)) {
      lo = 0.0;
      return ::log(x);
    }
    // |x - 1| < NEAR1, i.e. 1 - 2^-7 < x < 1 + 2^-7 (x - 1 is exact there, Sterbenz)
    if (bits > 0x3FEFC00000000000ll && bits < 0x3FF0200000000000ll) {
      lo = 0.0;
      return log1p_near1(x - 1.0);
    }
    const long long u = bits - 0x3FE8000000000000ll;       // relative to 0.75
    const long long e = u >> 52;                            // arithmetic shift
    const int j = (int)((u >> 44) & (FM_LOG_N - 1));
    const double m = __longlong_as_double(bits - (e << 52));
    const double r = __fma_rn(m, log_ic[j], -1.0);
    const double b = log1p_poly(r);
    const double ed = (double)e;
    const double ln2_hi = 0.6931471805598903;               // 42 significant bits
    const double ln2_lo = 5.497923018708371e-14;            // ln 2 - ln2_hi
    const double t1 = __dmul_rn(ed, ln2_hi);                // exact
    const double a = __dadd_rn(t1, log_c[j]);
    const double ea = __dadd_rn(__dadd_rn(t1, -a), log_c[j]);   // |t1| >= |log_c| or t1 == 0
    const double hi = __dadd_rn(a, b);
    const double eb = __dadd_rn(b, -__dadd_rn(hi, -a));
    lo = __fma_rn(ed, ln2_lo, __dadd_rn(ea, eb));
    return hi;
  }

  // Near x = 1 the table split cancels; log(x) = log1p(f) with f = x - 1 is
  // evaluated directly as f + f^2 (-1/2 + f (1/3 + ... + f (-1/8))), whose
  // truncation error is below 2e-18 relative for |f| < 1/128.
  static constexpr double NEAR1 = 0.0078125;
  __device__ __forceinline__ static double log1p_near1(double f) {
    double q = __fma_rn(f, -1.2500000000000000e-01, 1.4285714285714285e-01);
    q = __fma_rn(q, f, -1.6666666666666666e-01);
    q = __fma_rn(q, f, 2.0e-01);
    q = __fma_rn(q, f, -0.25);
    q = __fma_rn(q, f, 3.3333333333333331e-01);
    q = __fma_rn(q, f, -0.5);
    return __fma_rn(q, __dmul_rn(f, f), f);
  }

  // log1p(r) = r - r^2/2 + r^3/3 - r^4/4 + r^5/5 - r^6/6 for |r| < 2e-3.
  __device__ __forceinline__ static double log1p_poly(double r) {
    double q = __fma_rn(r, -1.6666666666666666e-01, 2.0e-01);
    q = __fma_rn(q, r, -0.25);
    q = __fma_rn(q, r, 3.3333333333333331e-01);
    q = __fma_rn(q, r, -0.5);
    return __fma_rn(q, __dmul_rn(r, r), r);
  }

  // log(x) = hi + lo of log_hl, rounded once: within about half an ulp.
  __device__ __forceinline__ double log(double x) const {
    double lo;
    const double hi = log_hl(x, lo);
    return __dadd_rn(hi, lo);
  }

  // x^y for x >= 0 (the only use here); x == 0 gives 0 for y > 0.
  __device__ __forceinline__ double pow(double x, double y) const {
    if (fp_is_zero(x)) return fp_gt(y, 0.0) ? 0.0 : ::pow(x, y);
    double lo;
    const double hi = log_hl(x, lo);
    const double ph = __dmul_rn(y, hi);
    const double pl = __fma_rn(y, lo, __fma_rn(y, hi, -ph));
    const double e = exp(ph);
    return __fma_rn(e, pl, e);
  }
};

// FP32 transcendentals of the mixed-precision path (CUDA's expf / logf /
// powf, within 2 ulp of FP32).
struct FloatMath {
  __device__ __forceinline__ float exp(float x) const { return ::expf(x); }
  __device__ __forceinline__ float log(float x) const { return ::logf(x); }
  __device__ __forceinline__ float pow(float x, float y) const { return ::powf(x, y); }
};

// Same interface on top of the CUDA math library (used to separate the
// effects of the fast transcendentals from everything else).
struct LibMath {
  __device__ __forceinline__ double exp(double x) const { return ::exp(x); }
  __device__ __forceinline__ double log(double x) const { return ::log(x); }
  __device__ __forceinline__ double pow(double x, double y) const { return ::pow(x, y); }
};

}  // namespace nsw6
