// Kokkos_Core.hpp -- a minimal host-only stand-in for the handful of Kokkos names the reference's
// src_cpp_kokkos_host sources use (View<T**/T****, LayoutLeft>, HostMirror, create_mirror_view,
// deep_copy, MDRangePolicy<Rank<3|4>>, parallel_for, parallel_reduce with Min/Max,
// KOKKOS_LAMBDA, initialize/finalize/fence).  Test infrastructure for the oracle build only.
//
// Kokkos 4.7.03 (the version the reference fetches at configure time) is not available offline.
// This file follows Kokkos's documented semantics for the subset: LayoutLeft means the first
// index is fastest; views are zero-initialised reference-counted handles; a host mirror of a host
// view aliases it; MDRangePolicy iterates the half-open box [begin, end); Min/Max reducers
// overwrite the bound variable with the reduction result.  Loop order never changes results here:
// every parallel_for writes disjoint elements and min/max are order independent.
#ifndef ORACLE_REFSHIM_KOKKOS_CORE_HPP_
#define ORACLE_REFSHIM_KOKKOS_CORE_HPP_

#include <algorithm>
#include <cfloat>
#include <cstddef>
#include <memory>
#include <string>
#include <utility>

#define KOKKOS_LAMBDA [=]

namespace Kokkos {

struct LayoutLeft {};

template <class DataType, class Layout = LayoutLeft>
class View;

template <class T>
class View<T**, LayoutLeft> {
 public:
  using HostMirror = View<T**, LayoutLeft>;
  View() = default;
  View(const std::string&, std::size_t n0, std::size_t n1) : n0_(n0), n1_(n1) {
    mem_ = std::shared_ptr<T[]>(new T[n0 * n1]());
  }
  T& operator()(std::size_t i0, std::size_t i1) const { return mem_[i0 + n0_ * i1]; }
  T* data() const { return mem_.get(); }
  std::size_t size() const { return n0_ * n1_; }

 private:
  std::shared_ptr<T[]> mem_;
  std::size_t n0_ = 0, n1_ = 0;
};

template <class T>
class View<T****, LayoutLeft> {
 public:
  using HostMirror = View<T****, LayoutLeft>;
  View() = default;
  View(const std::string&, std::size_t n0, std::size_t n1, std::size_t n2, std::size_t n3)
      : n0_(n0), n1_(n1), n2_(n2), n3_(n3) {
    mem_ = std::shared_ptr<T[]>(new T[n0 * n1 * n2 * n3]());
  }
  T& operator()(std::size_t i0, std::size_t i1, std::size_t i2, std::size_t i3) const {
    return mem_[i0 + n0_ * (i1 + n1_ * (i2 + n2_ * i3))];
  }
  T* data() const { return mem_.get(); }
  std::size_t size() const { return n0_ * n1_ * n2_ * n3_; }

 private:
  std::shared_ptr<T[]> mem_;
  std::size_t n0_ = 0, n1_ = 0, n2_ = 0, n3_ = 0;
};

template <class D, class L>
View<D, L> create_mirror_view(const View<D, L>& v) { return v; }

template <class D, class L>
void deep_copy(const View<D, L>& dst, const View<D, L>& src) {
  if (dst.data() != src.data()) std::copy(src.data(), src.data() + src.size(), dst.data());
}

template <unsigned N>
struct Rank {};

template <class R>
struct MDRangePolicy;

template <unsigned N>
struct MDRangePolicy<Rank<N>> {
  long b[N], e[N];
  MDRangePolicy(const int (&lo)[N], const int (&hi)[N]) {
    for (unsigned d = 0; d < N; d++) { b[d] = lo[d]; e[d] = hi[d]; }
  }
};

template <class F>
void parallel_for(const std::string&, const MDRangePolicy<Rank<3>>& p, const F& f) {
#pragma omp parallel for collapse(2) schedule(static)
  for (long i2 = p.b[2]; i2 < p.e[2]; i2++)
    for (long i1 = p.b[1]; i1 < p.e[1]; i1++)
      for (long i0 = p.b[0]; i0 < p.e[0]; i0++) f((int)i0, (int)i1, (int)i2);
}

template <class F>
void parallel_for(const std::string&, const MDRangePolicy<Rank<4>>& p, const F& f) {
#pragma omp parallel for collapse(2) schedule(static)
  for (long i3 = p.b[3]; i3 < p.e[3]; i3++)
    for (long i2 = p.b[2]; i2 < p.e[2]; i2++)
      for (long i1 = p.b[1]; i1 < p.e[1]; i1++)
        for (long i0 = p.b[0]; i0 < p.e[0]; i0++) f((int)i0, (int)i1, (int)i2, (int)i3);
}

template <class T>
struct Min {
  T& ref;
  explicit Min(T& r) : ref(r) {}
  static T identity() { return DBL_MAX; }
  static T join(T a, T b) { return std::min(a, b); }
};

template <class T>
struct Max {
  T& ref;
  explicit Max(T& r) : ref(r) {}
  static T identity() { return -DBL_MAX; }
  static T join(T a, T b) { return std::max(a, b); }
};

template <class F, class Red>
void parallel_reduce(const std::string&, const MDRangePolicy<Rank<3>>& p, const F& f, Red red) {
  double result = Red::identity();
#pragma omp parallel
  {
    double loc = Red::identity();
#pragma omp for collapse(2) schedule(static)
    for (long i2 = p.b[2]; i2 < p.e[2]; i2++)
      for (long i1 = p.b[1]; i1 < p.e[1]; i1++)
        for (long i0 = p.b[0]; i0 < p.e[0]; i0++) f((int)i0, (int)i1, (int)i2, loc);
#pragma omp critical
    result = Red::join(result, loc);
  }
  red.ref = result;
}

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}
inline void fence() {}

}  // namespace Kokkos

#endif
