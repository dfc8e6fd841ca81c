// fv_dual.hpp -- forward-mode dual numbers for the oracle's tangent-linear
// model. TEST INFRASTRUCTURE ONLY.
//
// Dual<V, K> carries a value of type V (float or double) and K directional
// derivatives in double. Every value is computed with V's own operations in
// the order the restatement writes them, so the value parts of a
// Sim<Dual<V, K>> run are bit for bit those of Sim<V> (the FP32 value parts
// are the FP32 oracle's trajectory, which the CUDA path reproduces). The
// derivative parts propagate the chain rule in double along that
// trajectory: the tangent-linear model of the discrete step, linearised
// where the forward run went. Comparisons and selects look at values only,
// so the derivative follows the branch the forward took (the reference's
// kernels are `template <typename TTT>`, apps/na/fv.h:7, 195, 383, 442, so
// they admit such a type too).
#pragma once

#include <cmath>

#include "../fivonagi_gb300/csrc/fv_math.h"

namespace fvo {

template <class V, int K> struct Dual {
  V v{};
  double d[K] = {};

  Dual() = default;
  Dual(double x) : v(V(x)) {}  // constants: V's rounding of x, no derivative
  Dual(float x) : v(V(x)) {}
  Dual(int x) : v(V(x)) {}
  static Dual of(V x) {
    Dual r;
    r.v = x;
    return r;
  }
  explicit operator double() const { return double(v); }
  explicit operator float() const { return float(v); }

  Dual &operator+=(const Dual &b) {
    v = v + b.v;
    for (int k = 0; k < K; ++k) d[k] += b.d[k];
    return *this;
  }
  Dual &operator-=(const Dual &b) {
    v = v - b.v;
    for (int k = 0; k < K; ++k) d[k] -= b.d[k];
    return *this;
  }
};

template <class V, int K> inline Dual<V, K> operator-(const Dual<V, K> &a) {
  Dual<V, K> r;
  r.v = -a.v;
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <class V, int K> inline Dual<V, K> operator+(const Dual<V, K> &a, const Dual<V, K> &b) {
  Dual<V, K> r;
  r.v = a.v + b.v;
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <class V, int K> inline Dual<V, K> operator-(const Dual<V, K> &a, const Dual<V, K> &b) {
  Dual<V, K> r;
  r.v = a.v - b.v;
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <class V, int K> inline Dual<V, K> operator*(const Dual<V, K> &a, const Dual<V, K> &b) {
  Dual<V, K> r;
  r.v = a.v * b.v;
  const double av = double(a.v), bv = double(b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * bv + av * b.d[k];
  return r;
}
template <class V, int K> inline Dual<V, K> operator/(const Dual<V, K> &a, const Dual<V, K> &b) {
  Dual<V, K> r;
  r.v = a.v / b.v;
  // (da - (a/b) db) / b: no b*b, which underflows for the tiny wave norms
  // of a decaying FP64 tail
  const double bv = double(b.v), q = double(a.v) / bv;
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - q * b.d[k]) / bv;
  return r;
}
template <class V, int K> inline bool operator<(const Dual<V, K> &a, const Dual<V, K> &b) { return a.v < b.v; }
template <class V, int K> inline bool operator>(const Dual<V, K> &a, const Dual<V, K> &b) { return a.v > b.v; }
template <class V, int K> inline bool operator<=(const Dual<V, K> &a, const Dual<V, K> &b) { return a.v <= b.v; }
template <class V, int K> inline bool operator>=(const Dual<V, K> &a, const Dual<V, K> &b) { return a.v >= b.v; }
template <class V, int K> inline bool operator==(const Dual<V, K> &a, const Dual<V, K> &b) { return a.v == b.v; }
template <class V, int K> inline bool operator!=(const Dual<V, K> &a, const Dual<V, K> &b) { return a.v != b.v; }

// Elementary functions: V's value (the same call the plain oracle makes),
// derivative from the calculus in double.
template <class V, int K> inline Dual<V, K> dsqrt(const Dual<V, K> &a) {
  Dual<V, K> r;
  r.v = std::sqrt(a.v);
  const double g = 0.5 / std::sqrt(double(a.v));
  for (int k = 0; k < K; ++k) r.d[k] = g * a.d[k];
  return r;
}
template <class V, int K> inline Dual<V, K> dfabs(const Dual<V, K> &a) {
  Dual<V, K> r;
  r.v = std::fabs(a.v);
  const double s = a.v < V(0) ? -1.0 : 1.0;
  for (int k = 0; k < K; ++k) r.d[k] = s * a.d[k];
  return r;
}
// f(a) with value fv (already computed in V) and derivative df (double)
template <class V, int K> inline Dual<V, K> dchain(V fv, double df, const Dual<V, K> &a) {
  Dual<V, K> r;
  r.v = fv;
  for (int k = 0; k < K; ++k) r.d[k] = df * a.d[k];
  return r;
}

}  // namespace fvo
