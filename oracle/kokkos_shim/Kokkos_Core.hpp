// Minimal host-only stand-in for the subset of the Kokkos API that the NICAM
// NSW6 microphysics reference uses, so that its unmodified sources compile with
// plain g++ as the test oracle and CPU baseline.  TEST INFRASTRUCTURE ONLY:
// nothing in the shipped library includes or links this file.
//
// Execution model:
//   * NSW6_SHIM_OPENMP undefined -> every parallel_for is a serial loop nest in
//     row-major order (last index fastest).  This is the deterministic "strict"
//     oracle: for the rctop/tctop write race in TagBigLoop
//     (mod_mp_nsw6.cpp:1579-1592) the k = kmax write wins.
//   * NSW6_SHIM_OPENMP defined   -> loop nests are `omp parallel for collapse`,
//     which is how the reference's Kokkos-OpenMP build runs (CPU baseline).
//
// Memory model: every View lives in host memory, is zero-filled on allocation
// (Kokkos' default, which the reference relies on, e.g. mod_vadv1d.cpp:407) and
// is a shared, reference-counted handle.  Mirrors alias their source, so
// deep_copy between a view and its mirror is a no-op, as in real Kokkos for
// host-accessible spaces.
#pragma once

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <limits>
#include <tuple>
#include <type_traits>
#include <utility>

#if defined(NSW6_SHIM_OPENMP)
#include <omp.h>
#endif

#define KOKKOS_LAMBDA [=]
#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline

namespace Kokkos {

// ----------------------------------------------------------------- spaces
struct HostSpace {};
struct CudaSpace {};
struct LayoutRight {};
struct LayoutStride {};
struct Static {};
struct Dynamic {};
template <class T> struct Schedule {};

struct OpenMP {
  int concurrency() const {
#if defined(NSW6_SHIM_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
  }
};
struct Serial : OpenMP {};
struct Cuda : OpenMP {};
using DefaultExecutionSpace = OpenMP;

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}
inline void fence() {}
inline void fence(const std::string&) {}
inline void print_configuration(std::ostream& os, bool = false) {
  os << "nsw6 Kokkos shim (host"
#if defined(NSW6_SHIM_OPENMP)
     << ", OpenMP"
#else
     << ", serial"
#endif
     << ")\n";
}

template <class... Args>
inline int printf(const char* fmt, Args... args) {
  return std::printf(fmt, args...);
}

// Device-side aborts (Newton non-convergence, mod_satadjust.cpp:756-764,
// 883-891) are recorded instead of terminating the host process, so the
// oracle driver can turn them into an error return.
namespace shim {
inline std::atomic<int>& abort_count() {
  static std::atomic<int> n{0};
  return n;
}
}  // namespace shim
inline void abort(const char* msg) {
  shim::abort_count().fetch_add(1);
  std::fprintf(stderr, "[kokkos-shim] abort: %s\n", msg);
}

class Timer {
  std::chrono::steady_clock::time_point t0_ = std::chrono::steady_clock::now();
 public:
  void reset() { t0_ = std::chrono::steady_clock::now(); }
  double seconds() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
  }
};

// ----------------------------------------------------------------- math
template <class A, class B>
KOKKOS_INLINE_FUNCTION auto min(A a, B b) -> typename std::common_type<A, B>::type {
  using T = typename std::common_type<A, B>::type;
  return (T(b) < T(a)) ? T(b) : T(a);
}
template <class A, class B>
KOKKOS_INLINE_FUNCTION auto max(A a, B b) -> typename std::common_type<A, B>::type {
  using T = typename std::common_type<A, B>::type;
  return (T(a) < T(b)) ? T(b) : T(a);
}
inline double abs(double x) { return std::fabs(x); }
inline int abs(int x) { return std::abs(x); }
inline double copysign(double x, double y) { return std::copysign(x, y); }
inline double sqrt(double x) { return std::sqrt(x); }
inline double exp(double x) { return std::exp(x); }
inline double log(double x) { return std::log(x); }
template <class A, class B>
inline double pow(A x, B y) { return std::pow(double(x), double(y)); }

// ----------------------------------------------------------------- ALL
namespace Impl {
struct ALL_t {
  constexpr const ALL_t& operator()() const { return *this; }
};
}  // namespace Impl
constexpr Impl::ALL_t ALL = Impl::ALL_t{};

template <class T, std::size_t N>
struct Array {
  T v[N];
  T& operator[](std::size_t i) { return v[i]; }
  const T& operator[](std::size_t i) const { return v[i]; }
};

// ----------------------------------------------------------------- View
namespace Impl {
template <class D> struct data_traits { using value_type = D; static constexpr int rank = 0; };
template <class D> struct data_traits<D*> {
  using value_type = typename data_traits<D>::value_type;
  static constexpr int rank = data_traits<D>::rank + 1;
};
}  // namespace Impl

template <class DataType, class... Props>
class View {
 public:
  using value_type = typename std::remove_const<typename Impl::data_traits<DataType>::value_type>::type;
  static constexpr int Rank = Impl::data_traits<DataType>::rank;
  static constexpr int rank = Rank;

  std::shared_ptr<value_type> owner_;
  value_type* ptr_ = nullptr;
  std::size_t ext_[4] = {1, 1, 1, 1};
  std::size_t str_[4] = {0, 0, 0, 0};

  View() = default;

  template <class... N,
            typename = typename std::enable_if<sizeof...(N) == std::size_t(Rank)>::type>
  explicit View(const std::string& /*label*/, N... n) {
    set_extents({std::size_t(n)...});
    const std::size_t cnt = span();
    owner_ = std::shared_ptr<value_type>(new value_type[cnt == 0 ? 1 : cnt](),
                                         std::default_delete<value_type[]>());
    ptr_ = owner_.get();
  }

  // Unmanaged view over caller storage (row-major, contiguous).
  template <class... N,
            typename = typename std::enable_if<sizeof...(N) == std::size_t(Rank)>::type>
  View(value_type* p, N... n) {
    set_extents({std::size_t(n)...});
    ptr_ = p;
  }

  template <class D2, class... P2>
  View(const View<D2, P2...>& o) {
    static_assert(View<D2, P2...>::Rank == Rank, "rank mismatch in View conversion");
    owner_ = o.owner_;
    ptr_ = o.ptr_;
    for (int i = 0; i < 4; ++i) { ext_[i] = o.ext_[i]; str_[i] = o.str_[i]; }
  }

  template <class I0>
  value_type& operator[](I0 i0) const { return ptr_[std::size_t(i0) * str_[0]]; }
  value_type& operator()() const { return ptr_[0]; }
  template <class I0>
  value_type& operator()(I0 i0) const { return ptr_[std::size_t(i0) * str_[0]]; }
  template <class I0, class I1>
  value_type& operator()(I0 i0, I1 i1) const {
    return ptr_[std::size_t(i0) * str_[0] + std::size_t(i1) * str_[1]];
  }
  template <class I0, class I1, class I2>
  value_type& operator()(I0 i0, I1 i1, I2 i2) const {
    return ptr_[std::size_t(i0) * str_[0] + std::size_t(i1) * str_[1] + std::size_t(i2) * str_[2]];
  }
  template <class I0, class I1, class I2, class I3>
  value_type& operator()(I0 i0, I1 i1, I2 i2, I3 i3) const {
    return ptr_[std::size_t(i0) * str_[0] + std::size_t(i1) * str_[1] + std::size_t(i2) * str_[2] +
                std::size_t(i3) * str_[3]];
  }

  int extent_int(int d) const { return int(ext_[d]); }
  std::size_t extent(int d) const { return ext_[d]; }
  value_type* data() const { return ptr_; }
  std::size_t span() const {
    std::size_t s = 1;
    for (int i = 0; i < Rank; ++i) s *= ext_[i];
    return s;
  }
  std::size_t size() const { return span(); }
  bool contiguous() const {
    std::size_t s = 1;
    for (int i = Rank - 1; i >= 0; --i) {
      if (ext_[i] > 1 && str_[i] != s) return false;
      s *= ext_[i];
    }
    return true;
  }

 private:
  void set_extents(std::initializer_list<std::size_t> n) {
    int i = 0;
    for (std::size_t v : n) ext_[i++] = v;
    std::size_t s = 1;
    for (int d = Rank - 1; d >= 0; --d) { str_[d] = s; s *= ext_[d]; }
  }
};

// ----------------------------------------------------------------- subview
namespace Impl {
template <class V>
struct sub_builder {
  std::size_t off = 0;
  std::size_t ext[4] = {1, 1, 1, 1};
  std::size_t str[4] = {0, 0, 0, 0};
  int r = 0;
  int d = 0;
  const V& v;
  explicit sub_builder(const V& v_) : v(v_) {}
  void add(const ALL_t&) { ext[r] = v.ext_[d]; str[r] = v.str_[d]; ++r; ++d; }
  template <class I>
  void add(I i) { off += std::size_t(i) * v.str_[d]; ++d; }
};
template <class T, int R> struct rank_type { using type = typename rank_type<T, R - 1>::type*; };
template <class T> struct rank_type<T, 0> { using type = T; };
template <class A> constexpr int is_all() { return std::is_same<typename std::decay<A>::type, ALL_t>::value ? 1 : 0; }
}  // namespace Impl

template <class D, class... P, class... Args>
auto subview(const View<D, P...>& v, Args... args) {
  using V = View<D, P...>;
  constexpr int R = (0 + ... + Impl::is_all<Args>());
  using T = typename V::value_type;
  View<typename Impl::rank_type<T, R>::type, LayoutStride, HostSpace> out;
  Impl::sub_builder<V> b(v);
  (b.add(args), ...);
  out.owner_ = v.owner_;
  out.ptr_ = v.ptr_ + b.off;
  for (int i = 0; i < 4; ++i) { out.ext_[i] = b.ext[i]; out.str_[i] = b.str[i]; }
  return out;
}

// ----------------------------------------------------------------- copies
template <class V>
V create_mirror_view(const V& v) { return v; }
template <class S, class V>
V create_mirror_view(const S&, const V& v) { return v; }
template <class S, class V>
V create_mirror_view_and_copy(const S&, const V& v) { return v; }

template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
  if (dst.ptr_ == src.ptr_) return;
  constexpr int R = View<D1, P1...>::Rank;
  std::size_t e[4] = {1, 1, 1, 1};
  for (int i = 0; i < R; ++i) e[i] = dst.ext_[i];
  for (std::size_t a = 0; a < e[0]; ++a)
    for (std::size_t b = 0; b < e[1]; ++b)
      for (std::size_t c = 0; c < e[2]; ++c)
        for (std::size_t d = 0; d < e[3]; ++d) {
          std::size_t od = a * dst.str_[0] + b * dst.str_[1] + c * dst.str_[2] + d * dst.str_[3];
          std::size_t os = a * src.str_[0] + b * src.str_[1] + c * src.str_[2] + d * src.str_[3];
          dst.ptr_[od] = src.ptr_[os];
        }
}
template <class D1, class... P1, class S,
          typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
void deep_copy(const View<D1, P1...>& dst, const S& val) {
  constexpr int R = View<D1, P1...>::Rank;
  std::size_t e[4] = {1, 1, 1, 1};
  for (int i = 0; i < R; ++i) e[i] = dst.ext_[i];
  for (std::size_t a = 0; a < e[0]; ++a)
    for (std::size_t b = 0; b < e[1]; ++b)
      for (std::size_t c = 0; c < e[2]; ++c)
        for (std::size_t d = 0; d < e[3]; ++d)
          dst.ptr_[a * dst.str_[0] + b * dst.str_[1] + c * dst.str_[2] + d * dst.str_[3]] =
              typename View<D1, P1...>::value_type(val);
}

// ----------------------------------------------------------------- policies
template <int N> struct Rank { static constexpr int rank = N; };

namespace Impl {
template <class T> struct is_rank : std::false_type {};
template <int N> struct is_rank<Kokkos::Rank<N>> : std::true_type {};
template <class T> struct is_sched : std::false_type {};
template <class T> struct is_sched<Kokkos::Schedule<T>> : std::true_type {};
template <class T> struct is_space {
  static constexpr bool value = std::is_same<T, OpenMP>::value || std::is_same<T, Serial>::value ||
                                std::is_same<T, Cuda>::value || std::is_same<T, HostSpace>::value;
};
// First template argument that is neither a Rank, a Schedule nor a space is the work tag.
template <class... P> struct find_tag { using type = void; };
template <class H, class... P> struct find_tag<H, P...> {
  using type = typename std::conditional<is_rank<H>::value || is_sched<H>::value || is_space<H>::value,
                                         typename find_tag<P...>::type, H>::type;
};
template <class T> struct rank_value { static constexpr int value = 0; };
template <int N> struct rank_value<Kokkos::Rank<N>> { static constexpr int value = N; };
template <class... P> struct find_rank { static constexpr int value = 1; };
template <class H, class... P> struct find_rank<H, P...> {
  static constexpr int value = is_rank<H>::value ? rank_value<H>::value : find_rank<P...>::value;
};
}  // namespace Impl

template <class... P>
struct RangePolicy {
  using work_tag = typename Impl::find_tag<P...>::type;
  std::int64_t b, e;
  template <class B, class E>
  RangePolicy(B b_, E e_) : b(std::int64_t(b_)), e(std::int64_t(e_)) {}
};

template <class... P>
struct MDRangePolicy {
  using work_tag = typename Impl::find_tag<P...>::type;
  static constexpr int R = Impl::find_rank<P...>::value;
  std::int64_t lo[R], hi[R];
  template <class LT, std::size_t LN, class UT, std::size_t UN>
  MDRangePolicy(const LT (&l)[LN], const UT (&u)[UN]) {
    static_assert(LN == std::size_t(R) && UN == std::size_t(R), "MDRangePolicy bounds rank");
    for (int i = 0; i < R; ++i) { lo[i] = std::int64_t(l[i]); hi[i] = std::int64_t(u[i]); }
  }
  MDRangePolicy(const Array<std::int64_t, R>& l, const Array<std::int64_t, R>& u) {
    for (int i = 0; i < R; ++i) { lo[i] = l[i]; hi[i] = u[i]; }
  }
};

namespace Impl {
template <class Tag, class F, class... I>
inline void invoke(const F& f, I... i) {
  if constexpr (std::is_void<Tag>::value) f(i...);
  else f(Tag(), i...);
}
}  // namespace Impl

template <class... P, class F>
void parallel_for(const RangePolicy<P...>& p, const F& f) {
  using Tag = typename RangePolicy<P...>::work_tag;
#if defined(NSW6_SHIM_OPENMP)
#pragma omp parallel for schedule(static)
#endif
  for (std::int64_t i = p.b; i < p.e; ++i) Impl::invoke<Tag>(f, std::size_t(i));
}

template <class... P, class F>
void parallel_for(const MDRangePolicy<P...>& p, const F& f) {
  using Pol = MDRangePolicy<P...>;
  using Tag = typename Pol::work_tag;
  if constexpr (Pol::R == 2) {
    const std::int64_t b0 = p.lo[0], e0 = p.hi[0], b1 = p.lo[1], e1 = p.hi[1];
#if defined(NSW6_SHIM_OPENMP)
#pragma omp parallel for collapse(2) schedule(static)
#endif
    for (std::int64_t i = b0; i < e0; ++i)
      for (std::int64_t j = b1; j < e1; ++j) Impl::invoke<Tag>(f, std::size_t(i), std::size_t(j));
  } else if constexpr (Pol::R == 3) {
    const std::int64_t b0 = p.lo[0], e0 = p.hi[0], b1 = p.lo[1], e1 = p.hi[1], b2 = p.lo[2], e2 = p.hi[2];
#if defined(NSW6_SHIM_OPENMP)
#pragma omp parallel for collapse(3) schedule(static)
#endif
    for (std::int64_t i = b0; i < e0; ++i)
      for (std::int64_t j = b1; j < e1; ++j)
        for (std::int64_t k = b2; k < e2; ++k)
          Impl::invoke<Tag>(f, std::size_t(i), std::size_t(j), std::size_t(k));
  } else {
    static_assert(Pol::R == 4, "MDRangePolicy rank 2..4 supported");
    for (std::int64_t i = p.lo[0]; i < p.hi[0]; ++i)
      for (std::int64_t j = p.lo[1]; j < p.hi[1]; ++j)
        for (std::int64_t k = p.lo[2]; k < p.hi[2]; ++k)
          for (std::int64_t l = p.lo[3]; l < p.hi[3]; ++l)
            Impl::invoke<Tag>(f, std::size_t(i), std::size_t(j), std::size_t(k), std::size_t(l));
  }
}

template <class Pol, class F>
void parallel_for(const std::string&, const Pol& p, const F& f) { parallel_for(p, f); }

// ----------------------------------------------------------------- reductions
template <class T, class S = HostSpace>
struct Min {
  T& ref;
  explicit Min(T& r) : ref(r) {}
};
template <class T, class S = HostSpace>
struct Max {
  T& ref;
  explicit Max(T& r) : ref(r) {}
};

namespace Impl {
template <class R> struct red;
template <> struct red<double&> {
  static double init() { return 0.0; }
  static void join(double& a, double b) { a += b; }
  static double& out(double& r) { return r; }
};
template <class T, class S> struct red<Min<T, S>> {
  static T init() { return std::numeric_limits<T>::max(); }
  static void join(T& a, T b) { a = (b < a) ? b : a; }
  static T& out(Min<T, S>& r) { return r.ref; }
};
template <class T, class S> struct red<Max<T, S>> {
  static T init() { return std::numeric_limits<T>::lowest(); }
  static void join(T& a, T b) { a = (a < b) ? b : a; }
  static T& out(Max<T, S>& r) { return r.ref; }
};
}  // namespace Impl

template <class W, class Tup, class... V>
void reduce_write_all(W& w, Tup&& t, V... v) {
  std::apply([&](auto&&... r) { (w(r, v), ...); }, t);
}

// Serial reduction over a rank-2/3 MDRangePolicy with any mix of a plain sum
// and Min/Max reducers (the only form the reference uses, mod_debug.cpp:374, 397).
template <class... P, class F, class... Red>
void parallel_reduce(const MDRangePolicy<P...>& p, const F& f, Red&&... reds) {
  using Pol = MDRangePolicy<P...>;
  auto acc = std::make_tuple(Impl::red<typename std::conditional<
      std::is_same<typename std::decay<Red>::type, double>::value, double&,
      typename std::decay<Red>::type>::type>::init()...);
  if constexpr (Pol::R == 2) {
    for (std::int64_t i = p.lo[0]; i < p.hi[0]; ++i)
      for (std::int64_t j = p.lo[1]; j < p.hi[1]; ++j)
        std::apply([&](auto&... a) { f(std::size_t(i), std::size_t(j), a...); }, acc);
  } else {
    for (std::int64_t i = p.lo[0]; i < p.hi[0]; ++i)
      for (std::int64_t j = p.lo[1]; j < p.hi[1]; ++j)
        for (std::int64_t k = p.lo[2]; k < p.hi[2]; ++k)
          std::apply([&](auto&... a) { f(std::size_t(i), std::size_t(j), std::size_t(k), a...); }, acc);
  }
  auto write = [&](auto&& r, auto v) {
    using RT = typename std::decay<decltype(r)>::type;
    if constexpr (std::is_same<RT, double>::value) r = v;
    else r.ref = v;
  };
  std::apply([&](auto... v) { reduce_write_all(write, std::forward_as_tuple(reds...), v...); }, acc);
}

}  // namespace Kokkos
