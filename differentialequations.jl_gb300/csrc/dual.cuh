// dual.cuh -- forward-mode dual numbers: the Jacobian of a runtime-compiled
// right-hand side (rtc.cu) when the user gives none.
//
// This stands in for the reference's default Jacobian of the Rosenbrock
// methods, ForwardDiff's dual numbers (AutoForwardDiff, test/qa/qa.jl:12).
// Dual<T, N> carries a value and N partial derivatives.  With u_c seeded as
// (u_c, e_c) and the parameters as constants, one evaluation of f on duals
// gives every row of J = df/du: J[r][c] = f(u)_r.d[c].  The arithmetic is the
// chain rule of each operation; the functions below cover the operations a
// right-hand side typically uses.  Operators and functions are hidden friends,
// so mixed expressions with plain scalars (2.0 * u[0], u[1] - 1) convert the
// scalar to a constant dual.
#pragma once
#include "common.cuh"

namespace gbde {

template <class T, int N>
struct Dual {
  T v;
  T d[N];
  GBDE_D Dual() {}
  // a constant: any scalar convertible to T (int, float, double, T itself)
  template <class S>
  GBDE_D Dual(const S& x) : v(T(x)) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = T(0);
  }

  friend GBDE_D Dual operator+(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
  }
  friend GBDE_D Dual operator-(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
  }
  friend GBDE_D Dual operator-(const Dual& a) {
    Dual r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
  }
  friend GBDE_D Dual operator+(const Dual& a) { return a; }
  friend GBDE_D Dual operator*(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
  }
  friend GBDE_D Dual operator/(const Dual& a, const Dual& b) {
    Dual r;
    const T q = a.v / b.v;
    r.v = q;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - q * b.d[i]) / b.v;
    return r;
  }
  friend GBDE_D Dual& operator+=(Dual& a, const Dual& b) { return a = a + b; }
  friend GBDE_D Dual& operator-=(Dual& a, const Dual& b) { return a = a - b; }
  friend GBDE_D Dual& operator*=(Dual& a, const Dual& b) { return a = a * b; }
  friend GBDE_D Dual& operator/=(Dual& a, const Dual& b) { return a = a / b; }
  friend GBDE_D bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
  friend GBDE_D bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
  friend GBDE_D bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
  friend GBDE_D bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }

  // y = g(a.v), dy = g'(a.v) da
  GBDE_D static Dual chain(const Dual& a, T y, T dg) {
    Dual r;
    r.v = y;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = dg * a.d[i];
    return r;
  }
  friend GBDE_D Dual exp(const Dual& a) {
    const T e = exp(a.v);
    return chain(a, e, e);
  }
  friend GBDE_D Dual log(const Dual& a) { return chain(a, log(a.v), T(1) / a.v); }
  friend GBDE_D Dual sqrt(const Dual& a) {
    const T s = sqrt(a.v);
    return chain(a, s, T(0.5) / s);
  }
  friend GBDE_D Dual sin(const Dual& a) { return chain(a, sin(a.v), cos(a.v)); }
  friend GBDE_D Dual cos(const Dual& a) { return chain(a, cos(a.v), -sin(a.v)); }
  friend GBDE_D Dual tanh(const Dual& a) {
    const T t = tanh(a.v);
    return chain(a, t, T(1) - t * t);
  }
  friend GBDE_D Dual fabs(const Dual& a) { return chain(a, fabs(a.v), a.v < T(0) ? T(-1) : T(1)); }
  // a^b for a constant exponent
  friend GBDE_D Dual pow(const Dual& a, T b) {
    const T y = pow(a.v, b);
    return chain(a, y, b * pow(a.v, b - T(1)));
  }
};

// J[r][c] = d f_r / d u_c at (u, p) by one dual evaluation of M::f.
template <class M, class T>
GBDE_D void dual_jacobian(T (*J)[M::N], const T* u, const T* p) {
  using D = Dual<T, M::N>;
  D ud[M::N], pd[M::NP], fd[M::N];
#pragma unroll
  for (int c = 0; c < M::N; ++c) {
    ud[c] = D(u[c]);
    ud[c].d[c] = T(1);
  }
#pragma unroll
  for (int k = 0; k < M::NP; ++k) pd[k] = D(p[k]);
  M::f(fd, ud, pd);
#pragma unroll
  for (int r = 0; r < M::N; ++r)
#pragma unroll
    for (int c = 0; c < M::N; ++c) J[r][c] = fd[r].d[c];
}

}  // namespace gbde
