// Decision-recording build of the C restatement (TEST INFRASTRUCTURE ONLY).
//
// Compiles oracle/nsw6_oracle.c with every `double` replaced by a number type
// that records, in program order, every discrete decision the reference
// algorithm takes: the outcome of each comparison (which covers min/max, the
// limiters, the threshold tests, the Newton convergence test and the
// departure-cell search), the sign that each copysign/fabs selects and the
// value of each float-to-integer conversion (the Bergeron table index and the
// departure-cell arithmetic of vadv1d_getflux_new).  Two runs with equal
// records take the same branch everywhere, so the step is one smooth function
// of its inputs on the segment between them (the tangent-linear and adjoint
// steps hold exactly these decisions fixed).  The derivative tests use it to
// certify their finite-difference points: a central difference is only
// compared with the adjoint where the records at p, p +- h and p +- h/4 all
// equal the record at p.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "nsw6_oracle.h"

namespace bsig {
// One entry per decision: code = site << 2 | kind << 1 | outcome (kind 0: a
// comparison or a selected sign, kind 1: a float-to-integer conversion),
// val = the compared difference a - b, the sign argument, or the integer, and
// mag = the larger magnitude of the compared operands (the scale of val).
std::vector<uint8_t> code;
std::vector<double> val, mag;
int site = 0;
inline void decide(bool outcome, double v, double m) {
  code.push_back(static_cast<uint8_t>((site << 2) | (outcome ? 1 : 0)));
  val.push_back(v);
  mag.push_back(m);
}
inline void integer(long long v) {
  code.push_back(static_cast<uint8_t>((site << 2) | 2));
  val.push_back(static_cast<double>(v));
  mag.push_back(std::fabs(static_cast<double>(v)));
}
inline double larger(double a, double b) { return std::fmax(std::fabs(a), std::fabs(b)); }
}  // namespace bsig

struct bd {
  double v;
  bd() = default;
  constexpr bd(double x) : v(x) {}
  explicit operator int() const { bsig::integer((int)v); return (int)v; }
  explicit operator long() const { bsig::integer((long)v); return (long)v; }
  explicit operator unsigned long() const { bsig::integer((long long)(unsigned long)v); return (unsigned long)v; }
};
inline bd operator+(bd a, bd b) { return bd(a.v + b.v); }
inline bd operator-(bd a, bd b) { return bd(a.v - b.v); }
inline bd operator*(bd a, bd b) { return bd(a.v * b.v); }
inline bd operator/(bd a, bd b) { return bd(a.v / b.v); }
inline bd operator-(bd a) { return bd(-a.v); }
inline bd operator+(bd a) { return a; }
inline bd& operator+=(bd& a, bd b) { a = a + b; return a; }
inline bd& operator-=(bd& a, bd b) { a = a - b; return a; }
inline bd& operator*=(bd& a, bd b) { a = a * b; return a; }
#define BSIG_CMP(OP)                                              \
  inline bool operator OP(bd a, bd b) {                           \
    const bool r = a.v OP b.v;                                    \
    bsig::decide(r, a.v - b.v, bsig::larger(a.v, b.v));           \
    return r;                                                     \
  }
BSIG_CMP(<)
BSIG_CMP(>)
BSIG_CMP(<=)
BSIG_CMP(>=)
BSIG_CMP(==)
BSIG_CMP(!=)
#undef BSIG_CMP
inline bd sqrt(bd a) { return bd(std::sqrt(a.v)); }
inline bd exp(bd a) { return bd(std::exp(a.v)); }
inline bd log(bd a) { return bd(std::log(a.v)); }
inline bd pow(bd a, bd b) { return bd(std::pow(a.v, b.v)); }
inline bd pow(bd a, double b) { return pow(a, bd(b)); }
template <class I, typename std::enable_if<std::is_integral<I>::value, int>::type = 0>
inline bd pow(bd a, I b) { return pow(a, bd((double)b)); }
inline bd pow(double a, bd b) { return pow(bd(a), b); }
inline bd copysign(bd a, bd b) {
  bsig::decide(std::signbit(b.v), b.v, std::fabs(b.v));
  return bd(std::copysign(a.v, b.v));
}
inline bd fabs(bd a) {
  bsig::decide(std::signbit(a.v), a.v, std::fabs(a.v));
  return bd(std::fabs(a.v));
}

#define double bd
#define NSW6O_SITE(n) (bsig::site = (n))
#define nsw6o_default_params nsw6ob_default_params
#define nsw6o_mp_driver nsw6ob_mp_driver
#define nsw6o_max_threads nsw6ob_max_threads
#define nsw6o_params nsw6ob_params
#define NSW6_ORACLE_H
typedef struct nsw6ob_params {
  bd beta_saut, qicrt_saut, Cr, Cs, Cg, ice_nuc, kk_aut;
} nsw6ob_params;
int nsw6ob_mp_driver(int gall, int kall, const bd* gz, const bd* gzh, const nsw6ob_params* p, bd* const* a, bd dt,
                     bd ct, int itelim, int* status);
void nsw6ob_default_params(nsw6ob_params* p);
int nsw6ob_max_threads(void);
#include "nsw6_oracle.c"
#undef double

extern "C" {
// Runs one step in place (arrays as for nsw6o_mp_driver, parameters in the
// order of nsw6o_params) and records its decisions; returns the step's status
// and the number of decisions, which nsw6o_branch_copy then copies out.
int nsw6o_branch_record(int gall, int kall, const double* gz, const double* gzh, const double* p7, double* const* a,
                        double dt, long long* length) {
  bsig::code.clear();
  bsig::val.clear();
  bsig::mag.clear();
  bsig::site = 0;
  nsw6ob_params p;
  p.beta_saut = p7[0]; p.qicrt_saut = p7[1]; p.Cr = p7[2]; p.Cs = p7[3]; p.Cg = p7[4];
  p.ice_nuc = p7[5]; p.kk_aut = p7[6];
  int st[4];
  const int rc = nsw6ob_mp_driver(gall, kall, reinterpret_cast<const bd*>(gz), reinterpret_cast<const bd*>(gzh), &p,
                                  reinterpret_cast<bd* const*>(a), bd(dt), bd(0.0), 100, st);
  *length = static_cast<long long>(bsig::code.size());
  return rc;
}

void nsw6o_branch_copy(uint8_t* code, double* val, double* mag, long long n) {
  const size_t m = std::min(static_cast<size_t>(n), bsig::code.size());
  std::memcpy(code, bsig::code.data(), m);
  std::memcpy(val, bsig::val.data(), m * sizeof(double));
  std::memcpy(mag, bsig::mag.data(), m * sizeof(double));
}
}
