// rosenbrock.cuh -- Rosenbrock23, Rodas5 and Rodas5P single-trajectory
// steppers with an analytic Jacobian and an in-register LU of the small
// W-matrix.
//
// These replace OrdinaryDiffEq's Rosenbrock perform_step! (Rosenbrock23
// qa.jl:98, Rodas5P qa.jl:97; Rodas5P is the method of the stiff test at
// test/core.jl:38-49 and of the precompile workload at
// src/DifferentialEquations.jl:27-28), whose W-matrix is the
// WOperator / StaticWOperator of qa.jl:129,113 and whose LU the reference
// delegates to LinearSolve.  W and its LU are FP64 in both precision modes.
#pragma once
#include "ff.cuh"
#include "solver.cuh"
#include "tableaus.h"

namespace gbde {

// max over rows of sum_c |J_rc| in FP64, columns in order (the stiffness
// estimate of the Rosenbrock methods in a composite: Hairer & Wanner II, IV.2)
template <int N, class T>
GBDE_D double jac_inf_norm(const T (*J)[N]) {
  double mx = 0.0;
  bool nan = false;
#pragma unroll
  for (int r = 0; r < N; ++r) {
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < N; ++c) s += fabs((double)J[r][c]);
    nan |= s != s;
    mx = fmax(mx, s);
  }
  return nan ? __longlong_as_double(0x7ff8000000000000ll) : mx;
}

// ---------------------------------------------------------------- LU
// Partial-pivot LU of an N x N matrix held in registers.  Row swaps are done
// with compile-time indices and selects so that nothing spills to local
// memory; the reciprocal pivots (Newton-refined, controller.h) are kept for
// the triangular solves, and the pivot search compares magnitudes as
// integers.
template <int N>
struct SmallLU {
  double A[N][N];
  double inv[N];
  int piv[N];

  GBDE_HD void factor() {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      int pk = k;
      uint64_t best = mag_bits(A[k][k]);
#pragma unroll
      for (int r = k + 1; r < N; ++r) {
        const uint64_t v = mag_bits(A[r][k]);
        if (v > best) {
          best = v;
          pk = r;
        }
      }
      piv[k] = pk;
#pragma unroll
      for (int r = k + 1; r < N; ++r) {
        const bool sw = (pk == r);
#pragma unroll
        for (int c = 0; c < N; ++c) {
          const double x = A[k][c], y = A[r][c];
          A[k][c] = sw ? y : x;
          A[r][c] = sw ? x : y;
        }
      }
      inv[k] = rcp64(A[k][k]);
#pragma unroll
      for (int r = k + 1; r < N; ++r) {
        const double l = A[r][k] * inv[k];
        A[r][k] = l;
#pragma unroll
        for (int c = k + 1; c < N; ++c) A[r][c] -= l * A[k][c];
      }
    }
  }

  // x = A^{-1} b in FP64 (b and x may alias).  factor() swaps whole rows,
  // multipliers included (P A = L U, as LAPACK's getrf), so every row swap is
  // applied to b before the forward substitution (getrs's order).
  GBDE_HD void solve(double* b) const {
#pragma unroll
    for (int k = 0; k < N; ++k) {
#pragma unroll
      for (int r = k + 1; r < N; ++r) {
        const bool sw = (piv[k] == r);
        const double x = b[k], y = b[r];
        b[k] = sw ? y : x;
        b[r] = sw ? x : y;
      }
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
#pragma unroll
      for (int r = k + 1; r < N; ++r) b[r] -= A[r][k] * b[k];
    }
#pragma unroll
    for (int k = N - 1; k >= 0; --k) {
      double s = b[k];
#pragma unroll
      for (int c = k + 1; c < N; ++c) s -= A[k][c] * b[c];
      b[k] = s * inv[k];
    }
  }

  template <class T>
  GBDE_HD void solve_t(const T* rhs, T* x) const {
    double b[N];
#pragma unroll
    for (int c = 0; c < N; ++c) b[c] = (double)rhs[c];
    solve(b);
#pragma unroll
    for (int c = 0; c < N; ++c) x[c] = (T)b[c];
  }
};

// The FP64 LU factors rounded to ff, with the triangular solves in ff
// arithmetic (the F32X2 precision: the factorisation stays FP64, each of the
// 3-8 solves per step runs on the FP32 pipe).
template <int N>
struct FFLU {
  ff A[N][N];
  ff inv[N];
  int piv[N];
  GBDE_D void from(const SmallLU<N>& W) {
#pragma unroll
    for (int r = 0; r < N; ++r) {
#pragma unroll
      for (int c = 0; c < N; ++c) A[r][c] = ff(W.A[r][c]);
      inv[r] = ff(W.inv[r]);
      piv[r] = W.piv[r];
    }
  }
  GBDE_D void solve_t(const ff* rhs, ff* x) const {
    ff b[N];
#pragma unroll
    for (int c = 0; c < N; ++c) b[c] = rhs[c];
    // every row swap first, then the substitutions (P A = L U, as SmallLU)
#pragma unroll
    for (int k = 0; k < N; ++k) {
#pragma unroll
      for (int r = k + 1; r < N; ++r) {
        const bool sw = (piv[k] == r);
        const ff xk = b[k], yr = b[r];
        b[k] = sw ? yr : xk;
        b[r] = sw ? xk : yr;
      }
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
#pragma unroll
      for (int r = k + 1; r < N; ++r) b[r] -= A[r][k] * b[k];
    }
#pragma unroll
    for (int k = N - 1; k >= 0; --k) {
      ff acc = b[k];
#pragma unroll
      for (int c = k + 1; c < N; ++c) acc -= A[k][c] * x[c];
      x[k] = acc * inv[k];
    }
  }
};

// W-matrix solver for a stepper in precision T: the FP64 LU itself, or its
// ff copy for T = ff.
template <int N, class T>
struct WSolver {
  SmallLU<N> W;  // a register copy (no address of the factor escapes)
  GBDE_D void setup(const SmallLU<N>& w) { W = w; }
  GBDE_D void solve_t(const T* rhs, T* x) const { W.solve_t(rhs, x); }
};
template <int N>
struct WSolver<N, ff> {
  FFLU<N> L;
  GBDE_D void setup(const SmallLU<N>& w) { L.from(w); }
  GBDE_D void solve_t(const ff* rhs, ff* x) const { L.solve_t(rhs, x); }
};

// -------------------------------------------------------- Rosenbrock23
// Shampine & Reichelt (1997): W = I - h d J,
//   k1 = W^{-1} F0,  F1 = f(y0 + h/2 k1),  k2 = W^{-1}(F1 - k1) + k1,
//   y1 = y0 + h k2,  F2 = f(y1),
//   k3 = W^{-1}(F2 - e32 (k2 - F1) - 2 (k1 - F0)),  err = h/6 (k1 - 2 k2 + k3),
//   y(t0 + theta h) = y0 + h (theta(1-theta)/(1-2d) k1 + theta(theta-2d)/(1-2d) k2).
template <class M, class T>
struct Ros23Alg {
  static constexpr int ORDER = 2, ALG_ID = GBDE_ALG_ROSENBROCK23, N = M::N;
  T uu[N], un[N], F0[N], F2[N], k1[N], k2[N];
  T J[N][N];
  bool fresh;  // J valid for uu

  GBDE_D const T* u() const { return uu; }
  GBDE_D const T* unew() const { return un; }
  GBDE_D const T* f0() const { return F0; }

  GBDE_D void init(const T* u0, const T* p, int& nf) {
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = u0[c];
    M::f(F0, uu, p);
    ++nf;
    fresh = false;
  }
  // continue at u0 with f(u0) = f0 already known (a switch of methods)
  GBDE_D void init_from(const T* u0, const T* f0, const T*) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = u0[c];
      F0[c] = f0[c];
    }
    fresh = false;
  }
  // ||J||_inf of the Jacobian the last attempt used (stiffness estimate)
  GBDE_D double jac_norm() const { return jac_inf_norm<N>(J); }
  GBDE_D bool f0_valid() const { return true; }  // F0 = f(uu) after accept (F2)

  GBDE_D double attempt(double dt, const T* p, double abstol, double reltol, int& nf) {
    using namespace tab::ros23;
    if (!fresh) {
      M::jac(J, uu, p);
      fresh = true;
    }
    SmallLU<N> W;
    const double hd = dt * d;
#pragma unroll
    for (int r = 0; r < N; ++r)
#pragma unroll
      for (int c = 0; c < N; ++c) W.A[r][c] = (r == c ? 1.0 : 0.0) - hd * (double)J[r][c];
    W.factor();
    WSolver<N, T> S;
    S.setup(W);
    const T h = (T)dt;
    S.solve_t(F0, k1);
    T y[N], F1[N], r3[N], k3[N];
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = uu[c] + T(0.5) * h * k1[c];
    M::f(F1, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = F1[c] - k1[c];
    S.solve_t(y, k2);
#pragma unroll
    for (int c = 0; c < N; ++c) {
      k2[c] += k1[c];
      un[c] = uu[c] + h * k2[c];
    }
    M::f(F2, un, p);
    nf += 2;
#pragma unroll
    for (int c = 0; c < N; ++c)
      r3[c] = F2[c] - T(e32) * (k2[c] - F1[c]) - T(2) * (k1[c] - F0[c]);
    S.solve_t(r3, k3);
    T err[N];
    T h6;
    if constexpr (is_ff<T>::value) h6 = h * T(1.0 / 6.0);  // ff has no division
    else h6 = h / T(6);
#pragma unroll
    for (int c = 0; c < N; ++c) err[c] = h6 * (k1[c] - T(2) * k2[c] + k3[c]);
    return err_ms<N>(err, uu, un, abstol, reltol);
  }

  GBDE_D void interp(double th, double dt, T* out, const T*, int&) {
    using namespace tab::ros23;
    const double den = 1.0 / (1.0 - 2.0 * d);
    const T w1 = (T)(th * (1.0 - th) * den), w2 = (T)(th * (th - 2.0 * d) * den);
    const T h = (T)dt;
#pragma unroll
    for (int c = 0; c < N; ++c) out[c] = uu[c] + h * (w1 * k1[c] + w2 * k2[c]);
  }

  GBDE_D void accept(const T*, int&) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = un[c];
      F0[c] = F2[c];
    }
    fresh = false;
  }
};

// ------------------------------------------------------------ Rodas5(P)
// Transformed form (Hairer-Wanner IV.7 (7.4')), 8 stages, stiffly accurate:
//   (I/(h gamma) - J) u_i = f(y0 + sum_{j<i} a_ij u_j) + sum_{j<i} (C_ij/h) u_j
//   with a_7j = a_6j (j<6), a_76 = 1; a_8j = a_7j (j<7), a_87 = 1;
//   y1 = y0 + sum_{j<8} a_8j u_j + u_8,  error estimate = u_8.
template <class Tab>
struct RodasCoef;

struct Rodas5Tag {};
struct Rodas5PTag {};

#define GBDE_RODAS_COEF(TAG, NS, DNS, ID)                                             \
  template <>                                                                         \
  struct RodasCoef<TAG> {                                                             \
    static constexpr int ALG_ID = ID;                                                 \
    static constexpr double g = tab::NS::gamma;                                       \
    static constexpr double a21 = tab::NS::a21, a31 = tab::NS::a31, a32 = tab::NS::a32; \
    static constexpr double a41 = tab::NS::a41, a42 = tab::NS::a42, a43 = tab::NS::a43; \
    static constexpr double a51 = tab::NS::a51, a52 = tab::NS::a52, a53 = tab::NS::a53, \
                            a54 = tab::NS::a54;                                       \
    static constexpr double a61 = tab::NS::a61, a62 = tab::NS::a62, a63 = tab::NS::a63, \
                            a64 = tab::NS::a64, a65 = tab::NS::a65;                   \
    static constexpr double C21 = tab::NS::C21, C31 = tab::NS::C31, C32 = tab::NS::C32; \
    static constexpr double C41 = tab::NS::C41, C42 = tab::NS::C42, C43 = tab::NS::C43; \
    static constexpr double C51 = tab::NS::C51, C52 = tab::NS::C52, C53 = tab::NS::C53, \
                            C54 = tab::NS::C54;                                       \
    static constexpr double C61 = tab::NS::C61, C62 = tab::NS::C62, C63 = tab::NS::C63, \
                            C64 = tab::NS::C64, C65 = tab::NS::C65;                   \
    static constexpr double C71 = tab::NS::C71, C72 = tab::NS::C72, C73 = tab::NS::C73, \
                            C74 = tab::NS::C74, C75 = tab::NS::C75, C76 = tab::NS::C76; \
    static constexpr double C81 = tab::NS::C81, C82 = tab::NS::C82, C83 = tab::NS::C83, \
                            C84 = tab::NS::C84, C85 = tab::NS::C85, C86 = tab::NS::C86, \
                            C87 = tab::NS::C87;                                       \
    static constexpr double H2[7] = {tab::DNS::H2_1, tab::DNS::H2_2, tab::DNS::H2_3,  \
                                     tab::DNS::H2_4, tab::DNS::H2_5, tab::DNS::H2_6,  \
                                     tab::DNS::H2_7};                                 \
    static constexpr double H3[7] = {tab::DNS::H3_1, tab::DNS::H3_2, tab::DNS::H3_3,  \
                                     tab::DNS::H3_4, tab::DNS::H3_5, tab::DNS::H3_6,  \
                                     tab::DNS::H3_7};                                 \
    static constexpr double H4[7] = {tab::DNS::H4_1, tab::DNS::H4_2, tab::DNS::H4_3,  \
                                     tab::DNS::H4_4, tab::DNS::H4_5, tab::DNS::H4_6,  \
                                     tab::DNS::H4_7};                                 \
  };
GBDE_RODAS_COEF(Rodas5Tag, rodas5, rodas5d, GBDE_ALG_RODAS5)
GBDE_RODAS_COEF(Rodas5PTag, rodas5p, rodas5pd, GBDE_ALG_RODAS5P)
#undef GBDE_RODAS_COEF

template <class M, class T, class Tag>
struct RodasAlg {
  using K = RodasCoef<Tag>;
  static constexpr int ORDER = 4, ALG_ID = K::ALG_ID, N = M::N;
  T uu[N], un[N], F0[N];
  T s1[N], s2[N], s3[N], s4[N], s5[N], s6[N], s7[N];  // transformed stages u_1..u_7
  T J[N][N];
  bool fresh;  // F0 and J valid for uu

  GBDE_D const T* u() const { return uu; }
  GBDE_D const T* unew() const { return un; }
  GBDE_D const T* f0() const { return F0; }

  GBDE_D void init(const T* u0, const T* p, int& nf) {
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = u0[c];
    M::f(F0, uu, p);
    ++nf;
    M::jac(J, uu, p);
    fresh = true;
  }
  // continue at u0 with f(u0) = f0 already known (a switch of methods)
  GBDE_D void init_from(const T* u0, const T* f0, const T* p) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = u0[c];
      F0[c] = f0[c];
    }
    M::jac(J, uu, p);
    fresh = true;
  }
  // ||J||_inf of the Jacobian the last attempt used (stiffness estimate)
  GBDE_D double jac_norm() const { return jac_inf_norm<N>(J); }
  GBDE_D bool f0_valid() const { return fresh; }  // F0 is re-evaluated after an accept

  GBDE_D double attempt(double dt, const T* p, double abstol, double reltol, int& nf) {
    if (!fresh) {
      M::f(F0, uu, p);
      ++nf;
      M::jac(J, uu, p);
      fresh = true;
    }
    SmallLU<N> W;
    const double ih = rcp64(dt);
    const double dg = ih * (1.0 / K::g);
#pragma unroll
    for (int r = 0; r < N; ++r)
#pragma unroll
      for (int c = 0; c < N; ++c) W.A[r][c] = r == c ? dg - (double)J[r][c] : -(double)J[r][c];
    W.factor();
    WSolver<N, T> S;
    S.setup(W);
    // r_i = f(y_i) + (1/h) sum_j C_ij u_j, with 1/h applied once per stage
    const T iht = (T)ih;
    T y[N], fy[N], r[N], s8[N];
    // stage 1
    S.solve_t(F0, s1);
    // stage 2
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = uu[c] + T(K::a21) * s1[c];
    M::f(fy, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) r[c] = fy[c] + iht * (T(K::C21) * s1[c]);
    S.solve_t(r, s2);
    // stage 3
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = uu[c] + T(K::a31) * s1[c] + T(K::a32) * s2[c];
    M::f(fy, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) r[c] = fy[c] + iht * (T(K::C31) * s1[c] + T(K::C32) * s2[c]);
    S.solve_t(r, s3);
    // stage 4
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = uu[c] + T(K::a41) * s1[c] + T(K::a42) * s2[c] + T(K::a43) * s3[c];
    M::f(fy, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) r[c] = fy[c] + iht * (T(K::C41) * s1[c] + T(K::C42) * s2[c] + T(K::C43) * s3[c]);
    S.solve_t(r, s4);
    // stage 5
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = uu[c] + T(K::a51) * s1[c] + T(K::a52) * s2[c] + T(K::a53) * s3[c] +
             T(K::a54) * s4[c];
    M::f(fy, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      r[c] = fy[c] + iht * (T(K::C51) * s1[c] + T(K::C52) * s2[c] + T(K::C53) * s3[c] + T(K::C54) * s4[c]);
    S.solve_t(r, s5);
    // stage 6
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = uu[c] + T(K::a61) * s1[c] + T(K::a62) * s2[c] + T(K::a63) * s3[c] +
             T(K::a64) * s4[c] + T(K::a65) * s5[c];
    M::f(fy, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      r[c] = fy[c] + iht * (T(K::C61) * s1[c] + T(K::C62) * s2[c] + T(K::C63) * s3[c] + T(K::C64) * s4[c] + T(K::C65) * s5[c]);
    S.solve_t(r, s6);
    // stage 7: y = U_6 + u_6
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] += s6[c];
    M::f(fy, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      r[c] = fy[c] + iht * (T(K::C71) * s1[c] + T(K::C72) * s2[c] + T(K::C73) * s3[c] + T(K::C74) * s4[c] + T(K::C75) * s5[c] + T(K::C76) * s6[c]);
    S.solve_t(r, s7);
    // stage 8: y = U_7 + u_7
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] += s7[c];
    M::f(fy, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      r[c] = fy[c] + iht * (T(K::C81) * s1[c] + T(K::C82) * s2[c] + T(K::C83) * s3[c] + T(K::C84) * s4[c] + T(K::C85) * s5[c] + T(K::C86) * s6[c] + T(K::C87) * s7[c]);
    S.solve_t(r, s8);
    nf += 7;
#pragma unroll
    for (int c = 0; c < N; ++c) un[c] = y[c] + s8[c];
    return err_ms<N>(s8, uu, un, abstol, reltol);
  }

  // y(theta) = (1-theta) y0 + theta y1 + theta(1-theta)(K2 + theta K3 + theta^2 K4),
  // K_q = sum_j Hq_j u_j, evaluated as y0 + theta (y1 - y0) + sum_j e_j u_j with
  // the scalar weights e_j = theta(1-theta)(H2_j + theta H3_j + theta^2 H4_j):
  // one 7-term combination per component instead of three.
  GBDE_D void interp(double th, double, T* out, const T*, int&) {
    const double w = th * (1.0 - th);
    T e[7];
#define GBDE_RODAS_E(j)                                                        \
  {                                                                            \
    constexpr double h2 = K::H2[j], h3 = K::H3[j], h4 = K::H4[j];              \
    e[j] = (T)(w * (h2 + th * (h3 + th * h4)));                                \
  }
    GBDE_RODAS_E(0); GBDE_RODAS_E(1); GBDE_RODAS_E(2); GBDE_RODAS_E(3);
    GBDE_RODAS_E(4); GBDE_RODAS_E(5); GBDE_RODAS_E(6);
#undef GBDE_RODAS_E
    const T tt = (T)th;
#pragma unroll
    for (int c = 0; c < N; ++c)
      out[c] = uu[c] + tt * (un[c] - uu[c]) + (e[0] * s1[c] + e[1] * s2[c] + e[2] * s3[c] +
                                               e[3] * s4[c] + e[4] * s5[c] + e[5] * s6[c] +
                                               e[6] * s7[c]);
  }

  GBDE_D void accept(const T*, int&) {
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = un[c];
    fresh = false;
  }
};

}  // namespace gbde
