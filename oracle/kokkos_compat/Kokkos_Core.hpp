// Kokkos-API-compatible host shim — TEST INFRASTRUCTURE ONLY.
//
// Implements exactly the Kokkos surface that the reference's single-rank header
// (src/pore_extraction.hpp) uses, so that header compiles UNMODIFIED with g++ and serves as the
// parity oracle for this project's CUDA path. It is never linked into the product library.
//
// Surface covered: DefaultExecutionSpace (::memory_space, ::name, fence), HostSpace,
// MemoryTraits<Unmanaged>, View<T*,Mem[,Traits]> and rank-0 View<T,Mem> (labelled ctor
// zero-initialises, shallow reference-counted copies, extent, operator(), value_type, data),
// unmanaged host views from (ptr, n), deep_copy (view<-view, view<-scalar), create_mirror_view,
// subview + make_pair, RangePolicy / MDRangePolicy<Rank<3>> with an execution-space instance,
// parallel_for / parallel_scan / parallel_reduce(Max<int>), atomic_min / atomic_add /
// atomic_fetch_add, floor, round, KOKKOS_LAMBDA, KOKKOS_INLINE_FUNCTION.
//
// Two modes: serial (default) and OpenMP (define PNM_SHIM_OPENMP and compile with -fopenmp).
// MDRange iterates z-outer / x-inner (memory order of the x-fastest layout); the integer results
// of the reference do not depend on the iteration order, only the pore emission order and the
// FP64 atomic accumulation order do.
#ifndef PNM_KOKKOS_COMPAT_CORE_HPP
#define PNM_KOKKOS_COMPAT_CORE_HPP

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>
#ifdef PNM_SHIM_OPENMP
#include <omp.h>
#endif

#define KOKKOS_LAMBDA [=]
#define KOKKOS_INLINE_FUNCTION inline

namespace Kokkos {

struct HostSpace {};

struct DefaultExecutionSpace {
  using memory_space = HostSpace;
  static const char* name() {
#ifdef PNM_SHIM_OPENMP
    return "OpenMP";
#else
    return "Serial";
#endif
  }
  void fence() const {}
};

inline bool& shim_initialized() {
  static bool v = false;
  return v;
}
inline void initialize() { shim_initialized() = true; }
inline void finalize() {}
inline bool is_initialized() { return shim_initialized(); }
inline bool is_finalized() { return false; }

enum MemoryTraitsFlags : unsigned { Unmanaged = 1u };
template <unsigned F>
struct MemoryTraits {
  static constexpr unsigned flags = F;
};

using std::make_pair;

// ---- View ----------------------------------------------------------------------------------
// Primary template: rank-0 view (a single shared scalar).
template <class T, class... Props>
class View {
 public:
  using value_type = T;
  View() = default;
  explicit View(const std::string& /*label*/) : store_(std::make_shared<T>()) {}
  T& operator()() const { return *store_; }
  T* data() const { return store_.get(); }
  std::shared_ptr<T> store_;
};

template <class P>
struct is_unmanaged_trait : std::false_type {};
template <unsigned F>
struct is_unmanaged_trait<MemoryTraits<F>> : std::bool_constant<(F & Unmanaged) != 0> {};

// rank-1 view: shallow, reference-counted; the labelled constructor zero-initialises. The
// (pointer, size) constructor exists only for views declared with MemoryTraits<Unmanaged>.
template <class T, class... Props>
class View<T*, Props...> {
 public:
  using value_type = T;
  using non_const_value_type = typename std::remove_const<T>::type;

  View() = default;
  View(const std::string& /*label*/, std::size_t n) : n_(n) {
    auto* raw = new non_const_value_type[n ? n : 1]();
    store_ = std::shared_ptr<non_const_value_type>(raw, std::default_delete<non_const_value_type[]>());
    ptr_ = raw;
  }
  View(T* p, std::size_t n)
    requires((is_unmanaged_trait<Props>::value || ...))
      : ptr_(p), n_(n) {}

  T& operator()(std::size_t i) const { return ptr_[i]; }
  std::size_t extent(int) const { return n_; }
  std::size_t size() const { return n_; }
  T* data() const { return ptr_; }

  std::shared_ptr<non_const_value_type> store_;
  T* ptr_ = nullptr;
  std::size_t n_ = 0;
};

template <class D, class S>
inline void deep_copy(const D& dst, const S& src) {
  if constexpr (std::is_arithmetic<S>::value) {
    if constexpr (requires { dst.extent(0); }) {
      for (std::size_t i = 0; i < dst.extent(0); ++i) dst(i) = src;
    } else {
      dst() = src;
    }
  } else {
    if constexpr (requires { dst.extent(0); }) {
      const std::size_t n = std::min(dst.extent(0), src.extent(0));
      if (n) std::memmove((void*)dst.data(), (const void*)src.data(), n * sizeof(*src.data()));
    } else {
      dst() = src();
    }
  }
}

template <class V>
inline V create_mirror_view(const V& v) {
  return v;  // host memory space: the mirror is the view itself
}

template <class T, class... Props>
inline View<T*, Props...> subview(const View<T*, Props...>& v, std::pair<std::size_t, std::size_t> r) {
  View<T*, Props...> s;
  s.store_ = v.store_;
  s.ptr_ = v.ptr_ + r.first;
  s.n_ = r.second - r.first;
  return s;
}

// ---- policies --------------------------------------------------------------------------------
template <int N>
struct Rank {};

template <class Exec>
struct RangePolicy {
  RangePolicy(const Exec&, std::size_t b, std::size_t e) : begin(b), end(e) {}
  RangePolicy(std::size_t b, std::size_t e) : begin(b), end(e) {}
  std::size_t begin, end;
};

template <class Exec, class R>
struct MDRangePolicy {
  MDRangePolicy(const Exec&, std::initializer_list<int> lo, std::initializer_list<int> hi) {
    std::copy(lo.begin(), lo.end(), l);
    std::copy(hi.begin(), hi.end(), h);
  }
  int l[3], h[3];
};

template <class Exec, class F>
inline void parallel_for(const std::string&, const RangePolicy<Exec>& p, const F& f) {
#ifdef PNM_SHIM_OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (long long i = (long long)p.begin; i < (long long)p.end; ++i) f((std::size_t)i);
}

template <class Exec, class R, class F>
inline void parallel_for(const std::string&, const MDRangePolicy<Exec, R>& p, const F& f) {
#ifdef PNM_SHIM_OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
  for (int z = p.l[2]; z < p.h[2]; ++z)
    for (int y = p.l[1]; y < p.h[1]; ++y)
      for (int x = p.l[0]; x < p.h[0]; ++x) f(x, y, z);
}

template <class Exec, class F>
inline void parallel_scan(const std::string&, const RangePolicy<Exec>& p, const F& f) {
#ifdef PNM_SHIM_OPENMP
  const long long b = (long long)p.begin, e = (long long)p.end;
  const int nt = omp_get_max_threads();
  std::vector<int> part(nt + 1, 0);
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    const long long len = e - b, lo = b + len * t / nt, hi = b + len * (t + 1) / nt;
    int upd = 0;
    for (long long i = lo; i < hi; ++i) f((std::size_t)i, upd, false);
    part[t + 1] = upd;
#pragma omp barrier
#pragma omp single
    for (int k = 1; k <= nt; ++k) part[k] += part[k - 1];
    upd = part[t];
    for (long long i = lo; i < hi; ++i) f((std::size_t)i, upd, true);
  }
#else
  int upd = 0;
  for (std::size_t i = p.begin; i < p.end; ++i) f(i, upd, true);
#endif
}

template <class T>
struct Max {
  explicit Max(T& r) : ref(r) {}
  T& ref;
};

template <class Exec, class F, class T>
inline void parallel_reduce(const std::string&, const RangePolicy<Exec>& p, const F& f, Max<T> red) {
  T best = std::numeric_limits<T>::lowest();
#ifdef PNM_SHIM_OPENMP
#pragma omp parallel
  {
    T loc = std::numeric_limits<T>::lowest();
#pragma omp for schedule(static)
    for (long long i = (long long)p.begin; i < (long long)p.end; ++i) f((std::size_t)i, loc);
#pragma omp critical
    best = std::max(best, loc);
  }
#else
  for (std::size_t i = p.begin; i < p.end; ++i) f(i, best);
#endif
  red.ref = best;
}

// ---- atomics -----------------------------------------------------------------------------------
template <class T>
inline void atomic_min_impl(T* p, T v) {
  std::atomic_ref<T> a(*p);
  T cur = a.load(std::memory_order_relaxed);
  while (v < cur && !a.compare_exchange_weak(cur, v, std::memory_order_relaxed)) {
  }
}
template <class T, class U>
inline void atomic_min(T* p, U v) {
  atomic_min_impl<T>(p, static_cast<T>(v));
}
template <class T, class U>
inline void atomic_add(T* p, U v) {
  std::atomic_ref<T> a(*p);
  a.fetch_add(static_cast<T>(v), std::memory_order_relaxed);
}
template <class T, class U>
inline T atomic_fetch_add(T* p, U v) {
  std::atomic_ref<T> a(*p);
  return a.fetch_add(static_cast<T>(v), std::memory_order_relaxed);
}

// ---- math -----------------------------------------------------------------------------------
inline double floor(double x) { return std::floor(x); }
inline float floor(float x) { return std::floor(x); }
inline double round(double x) { return std::round(x); }
inline float round(float x) { return std::round(x); }

}  // namespace Kokkos

#endif  // PNM_KOKKOS_COMPAT_CORE_HPP
