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

static long long check(double a, double b) {
  long long bad = 0;
  bad += fp_lt(a, b) != (a < b);
  bad += fp_le(a, b) != (a <= b);
  bad += fp_gt(a, b) != (a > b);
  bad += fp_ge(a, b) != (a >= b);
  bad += fp_is_zero(a) != (a == 0.0);
  for (double c : {708.0, 1.0e-12, 0.0078125, 1.0e300})
    bad += fp_abs_lt(a, c) != (std::fabs(a) < c);
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
