// IEEE-754 double comparisons evaluated on the integer pipe.
//
// On GB300 an FP64 compare issues to the FP64 pipe, which completes about two
// operations per SM per cycle, while the integer pipe completes 64; the NSW6
// kernels are FP64-pipe bound, so their comparisons (min / max, thresholds,
// range checks) are computed from the bit patterns instead.  Each function
// returns exactly what the IEEE comparison returns for every pair of doubles:
// false when either operand is NaN, -0 equal to +0.
//
// For a non-NaN x with bits b (as a signed 64-bit integer), the key
// b ^ ((b >> 63) & 0x7FF...F) orders the doubles like the reals, except that
// -0 (key -1) sorts below +0 (key 0); the zero pair is tested separately.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define NSW6_FP_HD __host__ __device__ __forceinline__
#else
#define NSW6_FP_HD inline
#endif

namespace nsw6 {

constexpr long long FP_ABS = 0x7FFFFFFFFFFFFFFFll;   // all but the sign
constexpr long long FP_INF = 0x7FF0000000000000ll;   // +inf; larger magnitudes are NaN

NSW6_FP_HD long long fp_bits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

NSW6_FP_HD long long fp_key(long long b) { return b ^ ((b >> 63) & FP_ABS); }

// a < b
NSW6_FP_HD bool fp_lt(double a, double b) {
  const long long ia = fp_bits(a), ib = fp_bits(b);
  const long long ma = ia & FP_ABS, mb = ib & FP_ABS;
  const bool ordered = (ma <= FP_INF) & (mb <= FP_INF);
  const bool zeros = (ma | mb) == 0;
  return ordered & !zeros & (fp_key(ia) < fp_key(ib));
}

// a <= b
NSW6_FP_HD bool fp_le(double a, double b) {
  const long long ia = fp_bits(a), ib = fp_bits(b);
  const long long ma = ia & FP_ABS, mb = ib & FP_ABS;
  const bool ordered = (ma <= FP_INF) & (mb <= FP_INF);
  const bool zeros = (ma | mb) == 0;
  return ordered & (zeros | (fp_key(ia) <= fp_key(ib)));
}

NSW6_FP_HD bool fp_gt(double a, double b) { return fp_lt(b, a); }
NSW6_FP_HD bool fp_ge(double a, double b) { return fp_le(b, a); }

// |x| < c for a constant c > 0 (NaN: false)
NSW6_FP_HD bool fp_abs_lt(double x, double c) { return (fp_bits(x) & FP_ABS) < fp_bits(c); }

// x < c for a constant c > 0: every negative x and -0 below it, a positive x
// by its bits (NaN: false)
NSW6_FP_HD bool fp_lt_pos(double x, double c) {
  const long long b = fp_bits(x);
  return ((b & FP_ABS) <= FP_INF) & (b < fp_bits(c));
}

// max(x, c) as Kokkos::max, (x < c) ? c : x, for a constant c > 0
NSW6_FP_HD double fp_max_pos(double x, double c) { return fp_lt_pos(x, c) ? c : x; }

// x == 0 (either zero)
NSW6_FP_HD bool fp_is_zero(double x) { return (fp_bits(x) & FP_ABS) == 0; }

// x is +-inf or NaN (x * 0 != 0)
NSW6_FP_HD bool fp_not_finite(double x) { return (fp_bits(x) & FP_ABS) >= FP_INF; }

// x is a positive normal number (not zero, subnormal, infinite or NaN)
NSW6_FP_HD bool fp_pos_normal(double x) {
  const long long b = fp_bits(x);
  return (b >= 0x0010000000000000ll) & (b < FP_INF);
}

// ---- comparisons with constants and the min / max they select (the cell
// physics' thresholds, clamps and limiters).  c: a positive normal constant
// (lt_negc: a negative one).  Each returns what the IEEE comparison (and the
// Kokkos::min / max select, (b < a) ? b : a and (a < b) ? b : a) returns.

NSW6_FP_HD double fp_from_bits(long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

constexpr long long FP_SIGN = -0x7FFFFFFFFFFFFFFFll - 1;   // the sign bit; -0

NSW6_FP_HD bool is_one(double x) { return fp_bits(x) == 0x3FF0000000000000ll; }        // x == 1
NSW6_FP_HD bool is_nonneg(double x) {                                                    // x >= 0
  const long long b = fp_bits(x);
  return (b >= 0 && b <= FP_INF) || b == FP_SIGN;
}
NSW6_FP_HD bool is_zero(double x) { return fp_is_zero(x); }                              // x == 0
NSW6_FP_HD bool lt_z(double x) {                                                         // x < 0
  return (unsigned long long)fp_bits(x) - 0x8000000000000001ull < 0x7FF0000000000000ull;
}
NSW6_FP_HD bool gt_z(double x) {                                                         // x > 0
  const long long b = fp_bits(x);
  return b > 0 && b <= FP_INF;
}
NSW6_FP_HD bool ge_c(double x, double c) {                                               // x >= c
  const long long b = fp_bits(x);
  return b >= fp_bits(c) && b <= FP_INF;
}
NSW6_FP_HD bool gt_c(double x, double c) {                                               // x > c
  const long long b = fp_bits(x);
  return b > fp_bits(c) && b <= FP_INF;
}
NSW6_FP_HD bool le_c(double x, double c) {                                               // x <= c
  const long long b = fp_bits(x);
  return b <= fp_bits(c) && (b & FP_ABS) <= FP_INF;
}
NSW6_FP_HD bool lt_c(double x, double c) { return fp_lt_pos(x, c); }                     // x < c
NSW6_FP_HD bool lt_negc(double x, double c) {                                            // x < c, c < 0
  const long long b = fp_bits(x), m = b & FP_ABS;
  return b < 0 && m > (fp_bits(c) & FP_ABS) && m <= FP_INF;
}
NSW6_FP_HD double maxz(double x) { return lt_z(x) ? 0.0 : x; }                          // max(x, 0)
NSW6_FP_HD double maxc(double x, double c) { return fp_lt_pos(x, c) ? c : x; }          // max(x, c)
NSW6_FP_HD double minc(double x, double c) { return gt_c(x, c) ? c : x; }               // min(x, c)

// The limiters' d = max(q, 0) / dt (dt > 0, which the API enforces) is not
// negative: +-0, positive, +inf or NaN.  d < p exactly when p is positive and
// not NaN and d's magnitude bits are below p's; a < -d exactly when a is
// negative, not NaN and of larger magnitude.
NSW6_FP_HD bool lt_nn(double d, double p) {                                             // d < p
  const long long bp = fp_bits(p);
  return bp > 0 && bp <= FP_INF && (fp_bits(d) & FP_ABS) < bp;
}
NSW6_FP_HD double min_nn(double p, double d) { return lt_nn(d, p) ? d : p; }            // min(p, d)
NSW6_FP_HD bool lt_nd(double a, double d) {                                             // a < -d
  const long long ba = fp_bits(a), ma = ba & FP_ABS;
  return ba < 0 && ma > (fp_bits(d) & FP_ABS) && ma <= FP_INF;
}
NSW6_FP_HD double max_nd(double a, double d) {                                          // max(a, -d)
  return lt_nd(a, d) ? fp_from_bits(fp_bits(d) ^ FP_SIGN) : a;
}

// x + 0.0: -0 becomes +0, every other value stays (a NaN keeps its payload,
// where an FP64 addition gives the canonical NaN)
NSW6_FP_HD double plus_zero(double x) { return fp_bits(x) == FP_SIGN ? 0.0 : x; }

}  // namespace nsw6
