// models.cuh -- built-in right-hand sides f(u, p) and analytic Jacobians.
//
// These stand in for the in-place ODEFunction f!(du, u, p, t) of the
// reference (ODEFunction, test/qa/qa.jl:84).  All models are autonomous.
// Formulas:
//   LINEAR     du = a u                                  (test/core.jl:10)
//   LORENZ     du = [s(y-x), x(r-z)-y, xy-bz]            (test/core.jl:22-27)
//   ROBERTSON  du = [-k1 y1 + k3 y2 y3,
//                    k1 y1 - k2 y2^2 - k3 y2 y3,
//                    k2 y2^2]                            (test/core.jl:39-45)
//   VDP_RING8  x_i' = v_i,
//              v_i' = mu (1 - x_i^2) v_i - x_i + kappa (x_{i-1} - 2 x_i + x_{i+1})
//              on a ring of 8 oscillators, state [x0, v0, x1, v1, ...]
//   LOTKA_VOLTERRA (SDE) drift [a x - b x y, d x y - g y], noise sigma * u
#pragma once
#include "common.cuh"
#include "../../include/gbde.h"

namespace gbde {

// log10 of a positive parameter (clamped away from 0) for the learned
// predictor's features
GBDE_HD float flog10(double x) { return (float)log10(fmax(fabs(x), 1e-30)); }

// Learned-predictor features (mlp.cuh): 8 numbers per trajectory from its
// parameters, initial state and time span, defined per model below.

struct Linear {
  static constexpr int N = 1, NP = 1, ID = GBDE_MODEL_LINEAR;
  static constexpr int F_FLOPS = 1;
  template <class T> GBDE_HD static void f(T* du, const T* u, const T* p) { du[0] = p[0] * u[0]; }
  template <class T> GBDE_HD static void jac(T (*J)[1], const T* u, const T* p) { J[0][0] = p[0]; }
  GBDE_HD static void features(const double* p, const double* u0, double span, float* f) {
    f[0] = (float)p[0]; f[1] = (float)u0[0]; f[2] = flog10(span);
    f[3] = f[4] = f[5] = f[6] = f[7] = 0.0f;
  }
};

struct Lorenz {
  static constexpr int N = 3, NP = 3, ID = GBDE_MODEL_LORENZ;
  static constexpr int F_FLOPS = 11;  // 2 + 4 + 3 (+2 subtractions)
  template <class T> GBDE_HD static void f(T* du, const T* u, const T* p) {
    du[0] = p[0] * (u[1] - u[0]);
    du[1] = u[0] * (p[1] - u[2]) - u[1];
    du[2] = u[0] * u[1] - p[2] * u[2];
  }
  template <class T> GBDE_HD static void jac(T (*J)[3], const T* u, const T* p) {
    J[0][0] = -p[0]; J[0][1] = p[0]; J[0][2] = T(0);
    J[1][0] = p[1] - u[2]; J[1][1] = T(-1); J[1][2] = -u[0];
    J[2][0] = u[1]; J[2][1] = u[0]; J[2][2] = -p[2];
  }
  GBDE_HD static void features(const double* p, const double* u0, double span, float* f) {
    f[0] = flog10(p[0]); f[1] = flog10(p[1]); f[2] = flog10(p[2]);
    f[3] = (float)u0[0]; f[4] = (float)u0[1]; f[5] = (float)u0[2]; f[6] = flog10(span); f[7] = 0.0f;
  }
};

struct Robertson {
  static constexpr int N = 3, NP = 3, ID = GBDE_MODEL_ROBERTSON;
  static constexpr int F_FLOPS = 12;
  template <class T> GBDE_HD static void f(T* du, const T* u, const T* p) {
    T r1 = p[0] * u[0];
    T r2 = p[1] * u[1] * u[1];
    T r3 = p[2] * u[1] * u[2];
    du[0] = -r1 + r3;
    du[1] = r1 - r2 - r3;
    du[2] = r2;
  }
  template <class T> GBDE_HD static void jac(T (*J)[3], const T* u, const T* p) {
    J[0][0] = -p[0]; J[0][1] = p[2] * u[2]; J[0][2] = p[2] * u[1];
    J[1][0] = p[0]; J[1][1] = T(-2) * p[1] * u[1] - p[2] * u[2]; J[1][2] = -p[2] * u[1];
    J[2][0] = T(0); J[2][1] = T(2) * p[1] * u[1]; J[2][2] = T(0);
  }
  GBDE_HD static void features(const double* p, const double* u0, double span, float* f) {
    f[0] = flog10(p[0]); f[1] = flog10(p[1]); f[2] = flog10(p[2]);
    f[3] = (float)u0[0]; f[4] = (float)u0[1]; f[5] = (float)u0[2]; f[6] = flog10(span); f[7] = 0.0f;
  }
};

struct VdpRing8 {
  static constexpr int N = 16, NP = 2, ID = GBDE_MODEL_VDP_RING8;
  static constexpr int F_FLOPS = 8 * 9;
  template <class T> GBDE_HD static void f(T* du, const T* u, const T* p) {
    const T mu = p[0], ka = p[1];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const T x = u[2 * i], v = u[2 * i + 1];
      const T xl = u[2 * ((i + 7) & 7)], xr = u[2 * ((i + 1) & 7)];
      du[2 * i] = v;
      du[2 * i + 1] = mu * (T(1) - x * x) * v - x + ka * (xl - T(2) * x + xr);
    }
  }
  template <class T> GBDE_HD static void jac(T (*J)[16], const T* u, const T* p) {
    const T mu = p[0], ka = p[1];
#pragma unroll
    for (int r = 0; r < 16; ++r)
#pragma unroll
      for (int c = 0; c < 16; ++c) J[r][c] = T(0);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const T x = u[2 * i], v = u[2 * i + 1];
      J[2 * i][2 * i + 1] = T(1);
      J[2 * i + 1][2 * i] = T(-2) * mu * x * v - T(1) - T(2) * ka;
      J[2 * i + 1][2 * i + 1] = mu * (T(1) - x * x);
      J[2 * i + 1][2 * ((i + 7) & 7)] += ka;
      J[2 * i + 1][2 * ((i + 1) & 7)] += ka;
    }
  }
  // Team kernels (team.cuh): lane r owns component r; `sh.bcast(v, src)`
  // reads lane src's value of v.  f_lane returns f_r(u); jac_lane fills row r
  // of the Jacobian.  Only the components row r depends on are fetched.
  template <class T, class Sh>
  GBDE_D static void ring_neighbours(int r, T y, const Sh& sh, T& x, T& v, T& xl, T& xr) {
    const int e = r & ~1;
    x = sh.bcast(y, e);
    v = sh.bcast(y, e | 1);
    xl = sh.bcast(y, (e + 14) & 15);
    xr = sh.bcast(y, (e + 2) & 15);
  }
  template <class T, class Sh>
  GBDE_D static T f_lane(int r, T y, const T* p, const Sh& sh) {
    T x, v, xl, xr;
    ring_neighbours(r, y, sh, x, v, xl, xr);
    const T dv = p[0] * (T(1) - x * x) * v - x + p[1] * (xl - T(2) * x + xr);
    return (r & 1) ? dv : v;
  }
  // 8-lane teams (one oscillator per lane): lane l holds (x_l, v_l) in y[0],
  // y[1]; only the neighbours' positions are fetched.  Same arithmetic as
  // f_lane and f.
  template <class T, class Sh>
  GBDE_D static void f_osc(int l, const T* y, const T* p, const Sh& sh, T* dy) {
    const T x = y[0], v = y[1];
    const T xl = sh.bcast(x, (l + 7) & 7), xr = sh.bcast(x, (l + 1) & 7);
    dy[0] = v;
    dy[1] = p[0] * (T(1) - x * x) * v - x + p[1] * (xl - T(2) * x + xr);
  }
  // f_osc for FP32 pairs P as one unnormalised pair accumulation (Acc: set /
  // add / fma / get), the same value to pair precision:
  //   v' = mu v - (mu v x) x - x - 2 ka x + ka xl + ka xr
  // (two pair products, five accumulated terms and one renormalisation,
  // instead of five renormalised products and five sums).  2 ka is exact.
  template <class Acc, class P, class Sh>
  GBDE_D static void f_osc_acc(int l, const P* y, const P* p, const Sh& sh, P* dy) {
    const P x = y[0], v = y[1];
    const P xl = sh.bcast(x, (l + 7) & 7), xr = sh.bcast(x, (l + 1) & 7);
    const P mv = p[0] * v, ka = p[1], ka2n(-2.0f * ka.hi, -2.0f * ka.lo);
    Acc a;
    a.set(mv);
    a.fma(-(mv * x), x);
    a.add(-x);
    a.fma(ka2n, x);
    a.fma(ka, xl);
    a.fma(ka, xr);
    dy[0] = v;
    dy[1] = a.get();
  }
  // 8-lane teams: rows 2l (x_l' = v_l) and 2l + 1 (v_l') of W = dg I - J at
  // lane l's oscillator (x, v) = (y[0], y[1]) have the nonzeros
  //   W[2l][2l] = dg, W[2l][2l + 1] = -1,
  //   W[2l + 1][2l] = w10, W[2l + 1][2l + 1] = w11, W[2l + 1][2(l +- 1)] = -ka
  // (jac_lane's rows negated, dg added on the diagonal).
  template <class T>
  GBDE_D static void w_osc_nz(const T* y, const T* p, T dg, T& w10, T& w11) {
    const T mu = p[0], ka = p[1], x = y[0], v = y[1];
    w10 = T(2) * mu * x * v + T(1) + T(2) * ka;
    w11 = dg - mu * (T(1) - x * x);
  }
  // r = b - W x on rows 2l, 2l + 1 with W's nonzeros (w_osc_nz) as pairs P
  // and x FP32 values (the lane's components; its neighbours' first
  // components fetched), accumulated in Acc (a pair accumulator with set /
  // fma / add / get): the residual of an FP32 solve, for a step of iterative
  // refinement.
  template <class Acc, class P, class Sh>
  GBDE_D static void w_osc_residual(int l, P dg, P w10, P w11, P ka, const P* b, const float* x,
                                    const Sh& sh, P* r) {
    const float xl = sh.bcast(x[0], (l + 7) & 7), xr = sh.bcast(x[0], (l + 1) & 7);
    Acc a;
    a.set(b[0]);
    a.fma(-dg, P(x[0], 0.0f));
    a.add(P(x[1], 0.0f));
    r[0] = a.get();
    Acc c;
    c.set(b[1]);
    c.fma(-w10, P(x[0], 0.0f));
    c.fma(-w11, P(x[1], 0.0f));
    c.fma(ka, P(xl, 0.0f));
    c.fma(ka, P(xr, 0.0f));
    r[1] = c.get();
  }
  template <class T, class Sh>
  GBDE_D static void jac_lane(int r, T y, const T* p, const Sh& sh, T* Jr) {
    T x, v, xl, xr;
    ring_neighbours(r, y, sh, x, v, xl, xr);
    const T mu = p[0], ka = p[1];
    const int e = r & ~1;
    const bool odd = r & 1;
    const T dx = T(-2) * mu * x * v - T(1) - T(2) * ka, dvv = mu * (T(1) - x * x);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      T val = T(0);
      if (odd) {
        if (c == e) val = dx;
        if (c == e + 1) val = dvv;
        if (c == ((e + 14) & 15)) val += ka;
        if (c == ((e + 2) & 15)) val += ka;
      } else if (c == r + 1) {
        val = T(1);
      }
      Jr[c] = val;
    }
  }
  // mu, kappa, span and summaries of the oscillators' initial state
  GBDE_HD static void features(const double* p, const double* u0, double span, float* f) {
    double mx = 0.0, mv = 0.0, sx = 0.0, sv = 0.0, sm = 0.0;
    for (int i = 0; i < 8; ++i) {
      const double x = u0[2 * i], v = u0[2 * i + 1];
      mx = fmax(mx, fabs(x));
      mv = fmax(mv, fabs(v));
      sx += x * x;
      sv += v * v;
      sm += fabs(1.0 - x * x) * fabs(v);
    }
    f[0] = flog10(p[0]); f[1] = (float)p[1]; f[2] = flog10(span); f[3] = (float)mx;
    f[4] = (float)mv; f[5] = (float)(sx / 8); f[6] = (float)(sv / 8); f[7] = flog10(p[0] * sm / 8);
  }
  // Row r of the Jacobian (for the warp-cooperative Rosenbrock path).
  template <class T> GBDE_HD static T jac_entry(int r, int c, const T* u, const T* p) {
    const T mu = p[0], ka = p[1];
    const int i = r >> 1;
    if ((r & 1) == 0) return c == r + 1 ? T(1) : T(0);
    const T x = u[2 * i], v = u[2 * i + 1];
    T val = T(0);
    if (c == 2 * i) val = T(-2) * mu * x * v - T(1) - T(2) * ka;
    if (c == 2 * i + 1) val = mu * (T(1) - x * x);
    if (c == 2 * ((i + 7) & 7)) val += ka;
    if (c == 2 * ((i + 1) & 7)) val += ka;
    return val;
  }
};

struct LotkaVolterra {
  static constexpr int N = 2, NP = 5, ID = GBDE_MODEL_LOTKA_VOLTERRA;
  static constexpr int F_FLOPS = 7, G_FLOPS = 2;
  template <class T> GBDE_HD static void f(T* du, const T* u, const T* p) {
    const T xy = u[0] * u[1];
    du[0] = p[0] * u[0] - p[1] * xy;
    du[1] = p[3] * xy - p[2] * u[1];
  }
  // diagonal noise g(u) = sigma * u
  template <class T> GBDE_HD static void g(T* gu, const T* u, const T* p) {
    gu[0] = p[4] * u[0];
    gu[1] = p[4] * u[1];
  }
  template <class T> GBDE_HD static void jac(T (*J)[2], const T* u, const T* p) {
    J[0][0] = p[0] - p[1] * u[1]; J[0][1] = -p[1] * u[0];
    J[1][0] = p[3] * u[1]; J[1][1] = p[3] * u[0] - p[2];
  }
  GBDE_HD static void features(const double* p, const double* u0, double span, float* f) {
    f[0] = flog10(p[0]); f[1] = flog10(p[1]); f[2] = flog10(p[2]); f[3] = flog10(p[3]);
    f[4] = (float)p[4]; f[5] = (float)u0[0]; f[6] = (float)u0[1]; f[7] = flog10(span);
  }
};

}  // namespace gbde
