// Operation-counting build of the C restatement (TEST INFRASTRUCTURE ONLY).
//
// Compiles oracle/nsw6_oracle.c with every `double` replaced by a counting
// number type, to measure the reference algorithm's FP64 work per cell on a
// given state: additions/subtractions, multiplications, divisions, square
// roots, exp, log, pow and comparisons (min/max/copysign/relational), split
// into phase 1 (what the GPU cell kernel computes) and phase 2 (the column
// kernel).  Data-dependent work (Newton iterations, flux-integral trip counts)
// is counted as executed.  bench.py turns the counts into the algorithmic
// FP64 work of the roofline.
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "nsw6_oracle.h"

namespace opc {
enum { ADD, MUL, DIV, SQRT, EXP, LOG, POW, CMP, NOPS };
long long counts[4][NOPS];
int phase = 0;
inline void tick(int op) { ++counts[phase][op]; }
}  // namespace opc

struct cd {
  double v;
  cd() = default;
  constexpr cd(double x) : v(x) {}
  explicit operator int() const { return (int)v; }
  explicit operator long() const { return (long)v; }
  explicit operator unsigned long() const { return (unsigned long)v; }
};
inline cd operator+(cd a, cd b) { opc::tick(opc::ADD); return cd(a.v + b.v); }
inline cd operator-(cd a, cd b) { opc::tick(opc::ADD); return cd(a.v - b.v); }
inline cd operator*(cd a, cd b) { opc::tick(opc::MUL); return cd(a.v * b.v); }
inline cd operator/(cd a, cd b) { opc::tick(opc::DIV); return cd(a.v / b.v); }
inline cd operator-(cd a) { return cd(-a.v); }
inline cd operator+(cd a) { return a; }
inline cd& operator+=(cd& a, cd b) { a = a + b; return a; }
inline cd& operator-=(cd& a, cd b) { a = a - b; return a; }
inline cd& operator*=(cd& a, cd b) { a = a * b; return a; }
inline bool operator<(cd a, cd b) { opc::tick(opc::CMP); return a.v < b.v; }
inline bool operator>(cd a, cd b) { opc::tick(opc::CMP); return a.v > b.v; }
inline bool operator<=(cd a, cd b) { opc::tick(opc::CMP); return a.v <= b.v; }
inline bool operator>=(cd a, cd b) { opc::tick(opc::CMP); return a.v >= b.v; }
inline bool operator==(cd a, cd b) { opc::tick(opc::CMP); return a.v == b.v; }
inline bool operator!=(cd a, cd b) { opc::tick(opc::CMP); return a.v != b.v; }
inline cd sqrt(cd a) { opc::tick(opc::SQRT); return cd(std::sqrt(a.v)); }
inline cd exp(cd a) { opc::tick(opc::EXP); return cd(std::exp(a.v)); }
inline cd log(cd a) { opc::tick(opc::LOG); return cd(std::log(a.v)); }
inline cd pow(cd a, cd b) {
  // A constant integer exponent n is counted as the n - 1 products that
  // evaluate it (exponent 0: nothing); other exponents as one pow.
  const double n = b.v;
  if (n == std::floor(n) && n >= 0.0 && n <= 8.0) {
    for (int i = 1; i < (int)n; ++i) opc::tick(opc::MUL);
    return cd(std::pow(a.v, n));
  }
  opc::tick(opc::POW);
  return cd(std::pow(a.v, b.v));
}
inline cd pow(cd a, double b) { return pow(a, cd(b)); }
template <class I, typename std::enable_if<std::is_integral<I>::value, int>::type = 0>
inline cd pow(cd a, I b) { return pow(a, cd((double)b)); }
inline cd pow(double a, cd b) { return pow(cd(a), b); }
inline cd copysign(cd a, cd b) { opc::tick(opc::CMP); return cd(std::copysign(a.v, b.v)); }
inline cd fabs(cd a) { return cd(std::fabs(a.v)); }

#define double cd
#define NSW6O_PHASE(n) (opc::phase = (n))
#define nsw6o_default_params nsw6oc_default_params
#define nsw6o_mp_driver nsw6oc_mp_driver
#define nsw6o_max_threads nsw6oc_max_threads
#define nsw6o_params nsw6oc_params
#define NSW6_ORACLE_H
typedef struct nsw6oc_params {
  cd beta_saut, qicrt_saut, Cr, Cs, Cg, ice_nuc, kk_aut;
} nsw6oc_params;
int nsw6oc_mp_driver(int gall, int kall, const cd* gz, const cd* gzh, const nsw6oc_params* p, cd* const* a, cd dt,
                     cd ct, int itelim, int* status);
void nsw6oc_default_params(nsw6oc_params* p);
int nsw6oc_max_threads(void);
#include "nsw6_oracle.c"
#undef double

extern "C" {
// Runs one counted step in place (arrays as for nsw6o_mp_driver); fills
// out[4][8] with the per-phase counts of ADD MUL DIV SQRT EXP LOG POW CMP.
int nsw6o_count_ops(int gall, int kall, const double* gz, const double* gzh, const double* p7, double* const* a,
                    double dt, long long* out) {
  std::memset(opc::counts, 0, sizeof(opc::counts));
  opc::phase = 0;
  nsw6oc_params p;
  p.beta_saut = p7[0]; p.qicrt_saut = p7[1]; p.Cr = p7[2]; p.Cs = p7[3]; p.Cg = p7[4];
  p.ice_nuc = p7[5]; p.kk_aut = p7[6];
  int st[4];
  const int rc = nsw6oc_mp_driver(gall, kall, reinterpret_cast<const cd*>(gz), reinterpret_cast<const cd*>(gzh), &p,
                                  reinterpret_cast<cd* const*>(a), cd(dt), cd(0.0), 100, st);
  std::memcpy(out, opc::counts, sizeof(opc::counts));
  return rc;
}
}
