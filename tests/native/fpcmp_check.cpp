// Checks the integer-pipe double comparisons of nsw6_fpcmp.cuh against the
// hardware's IEEE comparisons: special values (zeros, subnormals, infinities,
// NaNs of both signs) pairwise, then random bit patterns and random nearby
// pairs.  Prints the number of mismatches and exits non-zero on any.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#include "nsw6_fpcmp.cuh"

using namespace nsw6;

static double from_bits(unsigned long long b) {
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
}

static unsigned long long bits(double x) {
  unsigned long long b;
  std::memcpy(&b, &x, sizeof b);
  return b;
}

// the same double (bit for bit), or both NaN
static bool same(double x, double y) { return bits(x) == bits(y) || (std::isnan(x) && std::isnan(y)); }

static long long check(double a, double b) {
  long long bad = 0;
  bad += fp_lt(a, b) != (a < b);
  bad += fp_le(a, b) != (a <= b);
  bad += fp_gt(a, b) != (a > b);
  bad += fp_ge(a, b) != (a >= b);
  bad += fp_is_zero(a) != (a == 0.0);
  for (double c : {708.0, 1.0e-12, 0.0078125, 1.0e300})
    bad += fp_abs_lt(a, c) != (std::fabs(a) < c);
  // the cell physics' comparisons with constants and the selects they make
  bad += lt_z(a) != (a < 0.0);
  bad += gt_z(a) != (a > 0.0);
  bad += is_one(a) != (a == 1.0);
  bad += is_nonneg(a) != (a >= 0.0);
  bad += is_zero(a) != (a == 0.0);
  bad += !same(maxz(a), (a < 0.0) ? 0.0 : a);
  bad += bits(plus_zero(a)) != bits(a + 0.0) && !std::isnan(a);
  for (double c : {1.0e-12, 1.0e-10, 1.0e-8, 1.0e-5, 1.0e-4, 2.220446e-16, 1.0, 10.0, 1.0e3, 1.0e6, 1.75e-4}) {
    bad += ge_c(a, c) != (a >= c);
    bad += gt_c(a, c) != (a > c);
    bad += le_c(a, c) != (a <= c);
    bad += lt_c(a, c) != (a < c);
    bad += fp_lt_pos(a, c) != (a < c);
    bad += !same(maxc(a, c), (a < c) ? c : a);
    bad += !same(minc(a, c), (c < a) ? c : a);
  }
  for (double c : {-0.1, -30.99, -1.0e-300})
    bad += lt_negc(a, c) != (a < c);
  // a limiter bound d = max(q, 0) / dt is not negative: b with its sign cleared
  double d = std::fabs(b);
  for (int s = 0; s < 2; ++s, d = std::isnan(b) ? -std::fabs(b) : (d == 0.0 ? -0.0 : d)) {
    bad += lt_nn(d, a) != (d < a);
    bad += !same(min_nn(a, d), (d < a) ? d : a);
    bad += lt_nd(a, d) != (a < -d);
    bad += !same(max_nd(a, d), (a < -d) ? -d : a);
  }
  return bad;
}

int main() {
  const double inf = std::numeric_limits<double>::infinity();
  std::vector<double> sp = {0.0, -0.0, 1.0, -1.0, 4.9e-324, -4.9e-324, 2.2250738585072014e-308,
                            -2.2250738585072014e-308, 1.7976931348623157e308, -1.7976931348623157e308,
                            inf, -inf, std::nan(""), -std::nan(""), from_bits(0x7FF0000000000001ull),
                            from_bits(0xFFF0000000000001ull), from_bits(0x7FFFFFFFFFFFFFFFull),
                            from_bits(0xFFFFFFFFFFFFFFFFull), 708.0, -708.0, std::nextafter(708.0, 0.0),
                            std::nextafter(708.0, 1e9), 1.0e-12, 1.0e-4, -1.0e-12, 0.5, 2.0};
  long long bad = 0, n = 0;
  for (double a : sp)
    for (double b : sp) {
      bad += check(a, b);
      ++n;
    }
  std::mt19937_64 rng(12345);
  for (int i = 0; i < 2000000; ++i) {
    const double a = from_bits(rng()), b = from_bits(rng());
    bad += check(a, b);
    // nearby pairs: same magnitude, a few ulps apart, either sign
    const unsigned long long base = rng() & 0x7FEFFFFFFFFFFFFFull;
    const double c = from_bits(base ^ ((rng() & 1) << 63));
    const double d = from_bits((base + (rng() % 5)) ^ ((rng() & 1) << 63));
    bad += check(c, d);
    n += 2;
  }
  std::printf("pairs %lld mismatches %lld\n", n, bad);
  return bad == 0 ? 0 : 1;
}
