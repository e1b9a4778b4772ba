// Derivative scalar types for the tangent-linear and adjoint kernels.
//
// The physics of the step is written once, as templates over its scalar type
// (nsw6_cell.cuh, nsw6_column_step.cuh).  Besides double and float it is
// instantiated with
//
//   Dual   forward mode: value and one tangent (the tangent-linear model);
//   RVar   reverse mode: value and the index of its node on a per-thread tape
//          that records, for every operation, its (at most two) operands and
//          the partial derivatives with respect to them; the adjoint sweep
//          walks the tape backwards (the adjoint model).
//
// Values are computed with exactly the operations of the FP64 kernels (the
// same fused multiply-adds, correctly rounded quotients and table-driven
// transcendentals), so a derivative instance follows the same trajectory as
// the plain step.  Branches (limiters, switches, min/max) follow the values;
// their derivative is the one of the branch taken, except that a rate clamped
// at zero (rate_on) is off where its argument is exactly zero.
#pragma once

#include <type_traits>

#include "nsw6_common.cuh"
#include "nsw6_fastmath.cuh"

namespace nsw6 {

// ------------------------------------------------------------------ Dual
struct Dual {
  double v, d;
  __device__ __forceinline__ Dual() : v(0.0), d(0.0) {}
  __device__ __forceinline__ Dual(double x) : v(x), d(0.0) {}
  __device__ __forceinline__ Dual(double x, double dx) : v(x), d(dx) {}
};

__device__ __forceinline__ Dual operator+(const Dual& a, const Dual& b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(const Dual& a, const Dual& b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator*(const Dual& a, const Dual& b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(const Dual& a, const Dual& b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator+(const Dual& a) { return a; }
__device__ __forceinline__ Dual& operator+=(Dual& a, const Dual& b) { return a = a + b; }
__device__ __forceinline__ Dual& operator-=(Dual& a, const Dual& b) { return a = a - b; }
__device__ __forceinline__ Dual& operator*=(Dual& a, const Dual& b) { return a = a * b; }
__device__ __forceinline__ bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
__device__ __forceinline__ bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
__device__ __forceinline__ bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
__device__ __forceinline__ bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }

__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(const Dual& x) { return x.v; }
__device__ __forceinline__ double val_of(const Dual& x) { return x.v; }
__device__ __forceinline__ Dual with_value(const Dual& x, double v) { return Dual(v, x.d); }
__device__ __forceinline__ double with_value(double, double v) { return v; }
// f(x) with value fv and derivative dfdx at x.
__device__ __forceinline__ Dual dep(double fv, const Dual& x, double dfdx) { return Dual(fv, dfdx * x.d); }
__device__ __forceinline__ Dual dep2(double fv, const Dual& x, double dx, const Dual& y, double dy) {
  return Dual(fv, dx * x.d + dy * y.d);
}

__device__ __forceinline__ Dual fmaR(const Dual& a, const Dual& b, const Dual& c) {
  return Dual(__fma_rn(a.v, b.v, c.v), a.d * b.v + a.v * b.d + c.d);
}
__device__ __forceinline__ Dual sqrtR(const Dual& x) {
  const double s = sqrt(x.v);
  return Dual(s, s > 0.0 ? 0.5 * x.d / s : 0.0);
}
__device__ __forceinline__ Dual fabsR(const Dual& x) { return x.v < 0.0 ? -x : x; }
__device__ __forceinline__ Dual dmin(const Dual& a, const Dual& b) { return (b < a) ? b : a; }
__device__ __forceinline__ Dual dmax(const Dual& a, const Dual& b) { return (a < b) ? b : a; }
__device__ __forceinline__ Dual rate_on(const Dual& x) { return x.v > 0.0 ? x : Dual(dmax(x.v, 0.0)); }
// The quotient helpers of the FP64 kernels give the correctly rounded a / b.
__device__ __forceinline__ Dual div_rn(const Dual& a, const Dual& b, const Dual&) { return a / b; }
__device__ __forceinline__ Dual sel(bool on, const Dual& x) { return on ? x : Dual(copysign(0.0, x.v)); }
__device__ __forceinline__ Dual per_dt(const Dual& q, const Dual& dt, const Dual&) { return q / dt; }

// ------------------------------------------------------------------ RVar
// The per-thread tape lives in global memory, interleaved over the threads of
// a launch (entry e of slot s at index e * nslot + s) so that a warp's tape
// traffic is coalesced.
struct Tape {
  int* pa;
  int* pb;
  double* da;
  double* db;
  double* adj;
  int nslot, slot, n, cap, overflow, count_only;
};

constexpr int AD_THREADS = 128;

__device__ __forceinline__ Tape& tape() {
  __shared__ Tape t[AD_THREADS];
  return t[threadIdx.x];
}

struct RVar {
  double v;
  int id;   // -1 for constants
  __device__ __forceinline__ RVar() : v(0.0), id(-1) {}
  __device__ __forceinline__ RVar(double x) : v(x), id(-1) {}
  __device__ __forceinline__ RVar(double x, int i) : v(x), id(i) {}
};

__device__ __forceinline__ RVar record(double v, int a, double da, int b, double db) {
  if (a < 0 && b < 0) return RVar(v);
  Tape& t = tape();
  if (t.count_only) return RVar(v, t.n++);   // sizing pass: count the entries only
  if (t.n >= t.cap) {
    t.overflow = 1;
    return RVar(v);
  }
  const size_t e = (size_t)t.n * t.nslot + t.slot;
  t.pa[e] = a;
  t.pb[e] = b;
  t.da[e] = da;
  t.db[e] = db;
  return RVar(v, t.n++);
}
// A new independent variable (its adjoint accumulates at the returned id).
__device__ __forceinline__ RVar leaf(double v) {
  Tape& t = tape();
  if (t.count_only) return RVar(v, t.n++);
  if (t.n >= t.cap) {
    t.overflow = 1;
    return RVar(v);
  }
  const size_t e = (size_t)t.n * t.nslot + t.slot;
  t.pa[e] = -1;
  t.pb[e] = -1;
  t.da[e] = 0.0;
  t.db[e] = 0.0;
  return RVar(v, t.n++);
}

__device__ __forceinline__ RVar operator+(const RVar& a, const RVar& b) { return record(a.v + b.v, a.id, 1.0, b.id, 1.0); }
__device__ __forceinline__ RVar operator-(const RVar& a, const RVar& b) { return record(a.v - b.v, a.id, 1.0, b.id, -1.0); }
__device__ __forceinline__ RVar operator*(const RVar& a, const RVar& b) { return record(a.v * b.v, a.id, b.v, b.id, a.v); }
__device__ __forceinline__ RVar operator/(const RVar& a, const RVar& b) {
  const double q = a.v / b.v;
  return record(q, a.id, 1.0 / b.v, b.id, -q / b.v);
}
__device__ __forceinline__ RVar operator-(const RVar& a) { return record(-a.v, a.id, -1.0, -1, 0.0); }
__device__ __forceinline__ RVar operator+(const RVar& a) { return a; }
__device__ __forceinline__ RVar& operator+=(RVar& a, const RVar& b) { return a = a + b; }
__device__ __forceinline__ RVar& operator-=(RVar& a, const RVar& b) { return a = a - b; }
__device__ __forceinline__ RVar& operator*=(RVar& a, const RVar& b) { return a = a * b; }
__device__ __forceinline__ bool operator<(const RVar& a, const RVar& b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(const RVar& a, const RVar& b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<=(const RVar& a, const RVar& b) { return a.v <= b.v; }
__device__ __forceinline__ bool operator>=(const RVar& a, const RVar& b) { return a.v >= b.v; }
__device__ __forceinline__ bool operator==(const RVar& a, const RVar& b) { return a.v == b.v; }
__device__ __forceinline__ bool operator!=(const RVar& a, const RVar& b) { return a.v != b.v; }

__device__ __forceinline__ double val(const RVar& x) { return x.v; }
__device__ __forceinline__ double val_of(const RVar& x) { return x.v; }
__device__ __forceinline__ RVar with_value(const RVar& x, double v) { return RVar(v, x.id); }
__device__ __forceinline__ RVar dep(double fv, const RVar& x, double dfdx) { return record(fv, x.id, dfdx, -1, 0.0); }
__device__ __forceinline__ RVar dep2(double fv, const RVar& x, double dx, const RVar& y, double dy) {
  return record(fv, x.id, dx, y.id, dy);
}

__device__ __forceinline__ RVar fmaR(const RVar& a, const RVar& b, const RVar& c) {
  // a*b as its own node, then + c with the fused value of the FP64 kernels
  const RVar ab = record(a.v * b.v, a.id, b.v, b.id, a.v);
  return record(__fma_rn(a.v, b.v, c.v), ab.id, 1.0, c.id, 1.0);
}
__device__ __forceinline__ RVar sqrtR(const RVar& x) {
  const double s = sqrt(x.v);
  return record(s, x.id, s > 0.0 ? 0.5 / s : 0.0, -1, 0.0);
}
__device__ __forceinline__ RVar fabsR(const RVar& x) { return x.v < 0.0 ? -x : x; }
__device__ __forceinline__ RVar dmin(const RVar& a, const RVar& b) { return (b < a) ? b : a; }
__device__ __forceinline__ RVar dmax(const RVar& a, const RVar& b) { return (a < b) ? b : a; }
__device__ __forceinline__ RVar rate_on(const RVar& x) { return x.v > 0.0 ? x : RVar(dmax(x.v, 0.0)); }
__device__ __forceinline__ RVar div_rn(const RVar& a, const RVar& b, const RVar&) { return a / b; }
__device__ __forceinline__ RVar sel(bool on, const RVar& x) { return on ? x : RVar(copysign(0.0, x.v)); }
__device__ __forceinline__ RVar per_dt(const RVar& q, const RVar& dt, const RVar&) { return q / dt; }

// Reverse sweep of the calling thread's tape: propagates the adjoints seeded
// in adj[] from the last entry to the first.
__device__ __forceinline__ void tape_reverse() {
  Tape& t = tape();
  for (int e = t.n - 1; e >= 0; --e) {
    const size_t i = (size_t)e * t.nslot + t.slot;
    const double g = t.adj[i];
    if (g == 0.0) continue;
    const int a = t.pa[i], b = t.pb[i];
    if (a >= 0) t.adj[(size_t)a * t.nslot + t.slot] += t.da[i] * g;
    if (b >= 0) t.adj[(size_t)b * t.nslot + t.slot] += t.db[i] * g;
  }
}
__device__ __forceinline__ double& adj_of(const RVar& x) {
  Tape& t = tape();
  return t.adj[(size_t)x.id * t.nslot + t.slot];
}

// ------------------------------------------------------------------ math
// exp / log / pow of a derivative type: values from the table-driven FP64
// routines of the plain step, derivatives from their closed forms.
template <class T>
struct ADMath {
  FastMath fm;
  __device__ __forceinline__ T exp(const T& x) const {
    const double e = fm.exp(val(x));
    return dep(e, x, e);
  }
  __device__ __forceinline__ T log(const T& x) const { return dep(fm.log(val(x)), x, 1.0 / val(x)); }
  __device__ __forceinline__ T pow(const T& x, const T& y) const {
    const double xv = val(x), yv = val(y);
    const double p = fm.pow(xv, yv);
    if (!(xv > 0.0)) return dep2(p, x, 0.0, y, 0.0);
    if constexpr (std::is_same<T, Dual>::value) {
      // a constant exponent (every pow of the scheme): no d/dy term, no log
      if (y.d == 0.0) return Dual(p, (yv * p / xv) * x.d);
    }
    return dep2(p, x, yv * p / xv, y, p * fm.log(xv));
  }
};

}  // namespace nsw6
