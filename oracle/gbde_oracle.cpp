// gbde_oracle.cpp -- CPU FP64 oracle for the ensemble hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: the tests, the smoke
// check and the benchmark's CPU-baseline leg call it; the product library
// (libgbde.so) never links or calls it.
//
// It is an independent restatement of the per-trajectory solve that
// SciMLBase's EnsembleThreads maps over trajectories (EnsembleThreads,
// test/qa/qa.jl:56; solve qa.jl:192), for the methods named by the
// reference's API: Tsit5 (qa.jl:119; test/core.jl:14,32), Vern7 (qa.jl:126),
// Rosenbrock23 (qa.jl:98), Rodas5P (qa.jl:97; test/core.jl:47,
// src/DifferentialEquations.jl:28) and Rodas5, and for the SDE methods EM and
// SOSRI of StochasticDiffEq (SDEProblem qa.jl:103).  The reference's own
// implementations live in OrdinaryDiffEq v7 / SciMLBase v3 / StochasticDiffEq
// (Project.toml:6-18), which are neither vendored nor runnable here (no Julia
// runtime); the numeric pins are the order conditions of the coefficient
// tables (tableaus.h, tests/test_tableaus.py), analytic solutions, scipy
// solve_ivp references and the reference's pinned behaviours
// (test/core.jl:9-19, 21-36, 38-49, 90-96).
//
// Everything is FP64 scalar code with runtime state size n <= 16.  The
// EnsembleThreads-equivalent baseline splits trajectories over a
// std::thread pool (oracle_ensemble_solve's nthreads argument).
//
// Build: oracle/build_oracle.py (g++ -O2 -ffp-contract=off).
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/gbde.h"
#include "../differentialequations.jl_gb300/csrc/controller.h"
#include "../differentialequations.jl_gb300/csrc/tableaus.h"

namespace {

constexpr int NMAX = 16;
using Vec = double[NMAX];

// ------------------------------------------------------------- models
struct Model {
  int id, n, np;
};

void rhs(int id, const double* u, const double* p, double* du) {
  switch (id) {
    case GBDE_MODEL_LINEAR: du[0] = p[0] * u[0]; break;
    case GBDE_MODEL_LORENZ:  // test/core.jl:22-27
      du[0] = p[0] * (u[1] - u[0]);
      du[1] = u[0] * (p[1] - u[2]) - u[1];
      du[2] = u[0] * u[1] - p[2] * u[2];
      break;
    case GBDE_MODEL_ROBERTSON: {  // test/core.jl:39-45
      const double r1 = p[0] * u[0], r2 = p[1] * u[1] * u[1], r3 = p[2] * u[1] * u[2];
      du[0] = -r1 + r3;
      du[1] = r1 - r2 - r3;
      du[2] = r2;
      break;
    }
    case GBDE_MODEL_VDP_RING8:
      for (int i = 0; i < 8; ++i) {
        const double x = u[2 * i], v = u[2 * i + 1];
        const double xl = u[2 * ((i + 7) % 8)], xr = u[2 * ((i + 1) % 8)];
        du[2 * i] = v;
        du[2 * i + 1] = p[0] * (1.0 - x * x) * v - x + p[1] * (xl - 2.0 * x + xr);
      }
      break;
    case GBDE_MODEL_LOTKA_VOLTERRA:
      du[0] = p[0] * u[0] - p[1] * u[0] * u[1];
      du[1] = p[3] * u[0] * u[1] - p[2] * u[1];
      break;
  }
}

void noise(int id, const double* u, const double* p, double* g) {
  if (id == GBDE_MODEL_LOTKA_VOLTERRA) {
    g[0] = p[4] * u[0];
    g[1] = p[4] * u[1];
  }
}

// Jacobian by rows: J[r*n + c] = d f_r / d u_c
void jacobian(int id, int n, const double* u, const double* p, double* J) {
  for (int k = 0; k < n * n; ++k) J[k] = 0.0;
  switch (id) {
    case GBDE_MODEL_LINEAR: J[0] = p[0]; break;
    case GBDE_MODEL_LORENZ:
      J[0] = -p[0]; J[1] = p[0];
      J[3] = p[1] - u[2]; J[4] = -1.0; J[5] = -u[0];
      J[6] = u[1]; J[7] = u[0]; J[8] = -p[2];
      break;
    case GBDE_MODEL_ROBERTSON:
      J[0] = -p[0]; J[1] = p[2] * u[2]; J[2] = p[2] * u[1];
      J[3] = p[0]; J[4] = -2.0 * p[1] * u[1] - p[2] * u[2]; J[5] = -p[2] * u[1];
      J[7] = 2.0 * p[1] * u[1];
      break;
    case GBDE_MODEL_VDP_RING8:
      for (int i = 0; i < 8; ++i) {
        const double x = u[2 * i], v = u[2 * i + 1];
        const int r = 2 * i + 1;
        J[(2 * i) * n + 2 * i + 1] = 1.0;
        J[r * n + 2 * i] += -2.0 * p[0] * x * v - 1.0 - 2.0 * p[1];
        J[r * n + 2 * i + 1] += p[0] * (1.0 - x * x);
        J[r * n + 2 * ((i + 7) % 8)] += p[1];
        J[r * n + 2 * ((i + 1) % 8)] += p[1];
      }
      break;
    case GBDE_MODEL_LOTKA_VOLTERRA:
      J[0] = p[0] - p[1] * u[1]; J[1] = -p[1] * u[0];
      J[2] = p[3] * u[1]; J[3] = p[3] * u[0] - p[2];
      break;
  }
}

bool model_of(int id, Model& m) {
  switch (id) {
    case GBDE_MODEL_LINEAR: m = {id, 1, 1}; return true;
    case GBDE_MODEL_LORENZ: m = {id, 3, 3}; return true;
    case GBDE_MODEL_ROBERTSON: m = {id, 3, 3}; return true;
    case GBDE_MODEL_VDP_RING8: m = {id, 16, 2}; return true;
    case GBDE_MODEL_LOTKA_VOLTERRA: m = {id, 2, 5}; return true;
  }
  return false;
}

// ------------------------------------------------------ dense LU (n x n)
struct LU {
  int n;
  double A[NMAX * NMAX];
  int piv[NMAX];
  void factor() {
    for (int k = 0; k < n; ++k) {
      int pk = k;
      double best = std::fabs(A[k * n + k]);
      for (int r = k + 1; r < n; ++r)
        if (std::fabs(A[r * n + k]) > best) { best = std::fabs(A[r * n + k]); pk = r; }
      piv[k] = pk;
      if (pk != k)
        for (int c = 0; c < n; ++c) std::swap(A[k * n + c], A[pk * n + c]);
      for (int r = k + 1; r < n; ++r) {
        const double l = A[r * n + k] / A[k * n + k];
        A[r * n + k] = l;
        for (int c = k + 1; c < n; ++c) A[r * n + c] -= l * A[k * n + c];
      }
    }
  }
  // factor() swaps whole rows, multipliers included (P A = L U, LAPACK's
  // getrf), so the solve applies every row swap to b first and then
  // substitutes (getrs's order).
  void solve(const double* b, double* x) const {
    for (int c = 0; c < n; ++c) x[c] = b[c];
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(x[k], x[piv[k]]);
    for (int k = 0; k < n; ++k)
      for (int r = k + 1; r < n; ++r) x[r] -= A[r * n + k] * x[k];
    for (int k = n - 1; k >= 0; --k) {
      double s = x[k];
      for (int c = k + 1; c < n; ++c) s -= A[k * n + c] * x[c];
      x[k] = s / A[k * n + k];
    }
  }
};

// ---------------------------------------------------------- utilities
// Mean square of the scaled error, EEst^2 (accept iff <= 1).
double wrms(int n, const double* e, const double* u, const double* un, double at, double rt) {
  double s = 0.0;
  for (int c = 0; c < n; ++c) {
    const double sc = at + rt * std::fmax(std::fabs(u[c]), std::fabs(un[c]));
    s += (e[c] / sc) * (e[c] / sc);
  }
  return s / n;
}

// Controller arithmetic.  Mode 0 (the default) evaluates the step-size factor
// and the starting-step powers with the FP32 series of controller.h, the
// kernels' own arithmetic, so that the oracle takes the kernels' steps.  Mode 1
// (oracle_set_controller(1)) is the textbook FP64 form with pow() and sqrt()
// -- the PI controller of Hairer-Norsett-Wanner I, Sec. II.4 as OrdinaryDiffEq
// evaluates it -- used to measure how far the FP32 series moves the step
// sequence.  Process-wide; set it before a solve, not during one.
int g_ctl_pow64 = 0;

double hw_h0_pow64(double s0, double s1, double tspan) {
  double h0 = 1e-6;
  if (s0 >= 1e-10 && s1 >= 1e-10 && std::isfinite(s0) && std::isfinite(s1))
    h0 = 0.01 * (std::sqrt(s0) / std::sqrt(s1));
  return std::fmin(h0, tspan);
}

double hw_dt_pow64(double h0, double s1, double s2, double tspan, int order) {
  const double d1 = std::sqrt(s1), d2 = std::sqrt(s2) / h0;
  const double m = std::fmax(d1, d2);
  double h1;
  if (!(m * m > 1e-30)) h1 = std::fmax(1e-6, h0 * 1e-3);
  else if (!std::isfinite(m)) h1 = 0.0;
  else h1 = std::pow(0.01 / m, 1.0 / (order + 1));
  return std::fmin(std::fmin(100.0 * h0, h1), tspan);
}

// Per-trajectory controller memory: log2(qold) for the FP32 series, qold for
// the FP64 form.
struct CtlMem {
  float lqold;
  double qold;
};

// Hairer-Norsett-Wanner I, Sec. II.4 starting step: mean squares of the
// scaled u0, f0 and f(u0 + h0 f0) - f0; the powers go through the shared
// hw_h0 / hw_dt (controller.h), as in the kernels.
double init_dt(const Model& m, const double* u0, const double* f0, const double* p,
               double tspan, int order, double at, double rt, int& nf) {
  const int n = m.n;
  double s0 = 0, s1 = 0;
  for (int c = 0; c < n; ++c) {
    const double sc = at + std::fabs(u0[c]) * rt;
    s0 += (u0[c] / sc) * (u0[c] / sc);
    s1 += (f0[c] / sc) * (f0[c] / sc);
  }
  s0 /= n;
  s1 /= n;
  const double h0 = g_ctl_pow64 ? hw_h0_pow64(s0, s1, tspan) : gbde::hw_h0(s0, s1, tspan);
  Vec u1, f1;
  for (int c = 0; c < n; ++c) u1[c] = u0[c] + h0 * f0[c];
  rhs(m.id, u1, p, f1);
  ++nf;
  double s2 = 0;
  for (int c = 0; c < n; ++c) {
    const double sc = at + std::fabs(u0[c]) * rt;
    s2 += ((f1[c] - f0[c]) / sc) * ((f1[c] - f0[c]) / sc);
  }
  return g_ctl_pow64 ? hw_dt_pow64(h0, s1, s2 / n, tspan, order)
                     : gbde::hw_dt(h0, s1, s2 / n, tspan, order);
}

struct Ctl {  // controller constants (gbde_opts)
  double at, rt, qmin, qmax, gamma, beta1, beta2, qsmin, qsmax, qoldinit, dtmin, dtmax, dt0;
  int64_t maxiters;
  int adaptive;
  gbde::CtlK k;  // step-size factor constants (controller.h, shared with the kernels)
};

CtlMem ctl_start(const Ctl& C) { return CtlMem{C.k.lqoldinit, C.qoldinit}; }

// Accepted step with EEst^2 = E: the factor r of dt_new = h r.
double ctl_accept_r(const Ctl& C, double E, CtlMem& m) {
  if (!g_ctl_pow64) return (double)gbde::ctl_accept(C.k, E, m.lqold);
  const double eest = std::sqrt(E);
  double q = std::pow(eest, C.beta1) / std::pow(m.qold, C.beta2) / C.gamma;
  q = std::fmax(1.0 / C.qmax, std::fmin(1.0 / C.qmin, q));
  if (q >= C.qsmin && q <= C.qsmax) q = 1.0;
  m.qold = std::fmax(eest, C.qoldinit);
  return 1.0 / q;
}

// Rejected step: the factor r of dt_new = h r.
double ctl_reject_r(const Ctl& C, double E) {
  if (!g_ctl_pow64) return (double)gbde::ctl_reject(C.k, E);
  if (!std::isfinite(E)) return C.qmin;
  const double q = std::fmin(1.0 / C.qmin, std::pow(std::sqrt(E), C.beta1) / C.gamma);
  return 1.0 / q;
}

// ---------------------------------------------------------- one trajectory
struct Out {
  const gbde_problem* P;
  gbde_outputs* O;
  int64_t i;
  void save(int j, const double* v, int n) {
    const size_t base = ((size_t)i * P->n_save + j) * n;
    if (O->u_dtype == GBDE_F32)
      for (int c = 0; c < n; ++c) ((float*)O->u)[base + c] = (float)v[c];
    else
      for (int c = 0; c < n; ++c) ((double*)O->u)[base + c] = v[c];
  }
  double ts(int j) const {
    return P->save_kind == GBDE_SAVE_GRID ? P->saveat[j] : P->saveat[(size_t)i * P->n_save + j];
  }
};

// Method interface for the ODE driver (virtual-free: a switch on alg).
struct Stepper {
  int alg, n, id;
  const double* p;
  double u[NMAX], un[NMAX], f0[NMAX];
  double k[11][NMAX];  // stages (RK) or transformed stages (Rodas)
  double J[NMAX * NMAX];
  bool fresh, have11;
  double eig = 0.0;  // the last attempt's stiffness estimate (switching composites)

  void init(const double* u0, int& nf) {
    for (int c = 0; c < n; ++c) u[c] = u0[c];
    rhs(id, u, p, f0);
    ++nf;
    fresh = false;
    have11 = false;
    if (alg == GBDE_ALG_RODAS5 || alg == GBDE_ALG_RODAS5P) {
      jacobian(id, n, u, p, J);
      fresh = true;
    }
  }

  // ---- Tsit5 (Tsitouras 2011)
  double tsit5(double h, const Ctl& C, int& nf) {
    using namespace gbde::tab::tsit5;
    const double A[7][6] = {{0},
                            {a21},
                            {a31, a32},
                            {a41, a42, a43},
                            {a51, a52, a53, a54},
                            {a61, a62, a63, a64, a65},
                            {a71, a72, a73, a74, a75, a76}};
    const double bt[7] = {bt1, bt2, bt3, bt4, bt5, bt6, bt7};
    for (int c = 0; c < n; ++c) k[0][c] = f0[c];
    double y[NMAX], g6[NMAX];
    for (int s = 1; s < 7; ++s) {
      for (int c = 0; c < n; ++c) {
        double acc = 0.0;
        for (int j = 0; j < s; ++j) acc += A[s][j] * k[j][c];
        y[c] = u[c] + h * acc;
      }
      if (s == 5)
        for (int c = 0; c < n; ++c) g6[c] = y[c];
      if (s == 6)
        for (int c = 0; c < n; ++c) un[c] = y[c];
      rhs(id, y, p, k[s]);
    }
    nf += 6;
    // stiffness estimate (Hairer & Wanner II, IV.2, infinity norm): the
    // largest |(k7 - k6) / (y1 - g6)| over components, NaN if any is NaN
    {
      double mx = 0.0;
      bool nan = false;
      for (int c = 0; c < n; ++c) {
        const double r = std::fabs((k[6][c] - k[5][c]) / (un[c] - g6[c]));
        nan |= r != r;
        mx = std::fmax(mx, r);
      }
      eig = nan ? NAN : mx;
    }
    double e[NMAX];
    for (int c = 0; c < n; ++c) {
      double acc = 0.0;
      for (int j = 0; j < 7; ++j) acc += bt[j] * k[j][c];
      e[c] = h * acc;
    }
    return wrms(n, e, u, un, C.at, C.rt);
  }
  void tsit5_interp(double th, double h, double* out) {
    using namespace gbde::tab::tsit5;
    const double t2 = th * th;
    const double b[7] = {r11 * th * (th - r12) * (t2 - r13 * th + r14),
                         r21 * t2 * (t2 - r22 * th + r23),
                         r31 * t2 * (t2 - r32 * th + r33),
                         r41 * (th - r42) * (th - r43) * t2,
                         r51 * (th - r52) * (th - r53) * t2,
                         r61 * (th - r62) * (th - r63) * t2,
                         r71 * (th - r72) * (th - r73) * t2};
    for (int c = 0; c < n; ++c) {
      double acc = 0.0;
      for (int j = 0; j < 7; ++j) acc += b[j] * k[j][c];
      out[c] = u[c] + h * acc;
    }
  }

  // ---- Vern7 (Verner 2010) with the 5th-order extension over k1..k10, f(y1)
  double vern7(double h, const Ctl& C, int& nf) {
    using namespace gbde::tab::vern7;
    double A[10][9] = {};
    A[1][0] = a21;
    A[2][0] = a31; A[2][1] = a32;
    A[3][0] = a41; A[3][2] = a43;
    A[4][0] = a51; A[4][2] = a53; A[4][3] = a54;
    A[5][0] = a61; A[5][2] = a63; A[5][3] = a64; A[5][4] = a65;
    A[6][0] = a71; A[6][2] = a73; A[6][3] = a74; A[6][4] = a75; A[6][5] = a76;
    A[7][0] = a81; A[7][2] = a83; A[7][3] = a84; A[7][4] = a85; A[7][5] = a86; A[7][6] = a87;
    A[8][0] = a91; A[8][2] = a93; A[8][3] = a94; A[8][4] = a95; A[8][5] = a96; A[8][6] = a97;
    A[8][7] = a98;
    A[9][0] = a101; A[9][2] = a103; A[9][3] = a104; A[9][4] = a105; A[9][5] = a106;
    A[9][6] = a107;
    const double b[10] = {b1, 0, 0, b4, b5, b6, b7, b8, b9, 0};
    const double bh[10] = {bh1, 0, 0, bh4, bh5, bh6, bh7, 0, 0, bh10};
    for (int c = 0; c < n; ++c) k[0][c] = f0[c];
    double y[NMAX];
    for (int s = 1; s < 10; ++s) {
      for (int c = 0; c < n; ++c) {
        double acc = 0.0;
        for (int j = 0; j < s; ++j) acc += A[s][j] * k[j][c];
        y[c] = u[c] + h * acc;
      }
      rhs(id, y, p, k[s]);
    }
    nf += 9;
    double e[NMAX];
    for (int c = 0; c < n; ++c) {
      double a1 = 0.0, a2 = 0.0;
      for (int j = 0; j < 10; ++j) {
        a1 += b[j] * k[j][c];
        a2 += (b[j] - bh[j]) * k[j][c];
      }
      un[c] = u[c] + h * a1;
      e[c] = h * a2;
    }
    have11 = false;
    return wrms(n, e, u, un, C.at, C.rt);
  }
  // Vern7's 7th-order dense output (dense_coeffs.h, vern7l; Enright, Jackson,
  // Norsett, Thomsen, ACM TOMS 12 (1986) bootstrapping): f(t+h, y1) once per
  // step, then per save point three stages on the 5th-order extension and
  // four on the degree-6 interpolant through them;
  //   u(theta) = y0 + h sum_j (sum_m D_j_m theta^m) K_j,  j = 1..18.
  void vern7_interp(double th, double h, double* out, int& nf) {
    using namespace gbde::tab::vern7l;
    if (!have11) {
      rhs(id, un, p, k[10]);
      ++nf;
      have11 = true;
    }
#define GBDE_O_ROW11(P, i) {P##i##_1, P##i##_2, P##i##_3, P##i##_4, P##i##_5, P##i##_6, \
                            P##i##_7, P##i##_8, P##i##_9, P##i##_10, P##i##_11}
    const double L1[3][11] = {GBDE_O_ROW11(L1_, 1), GBDE_O_ROW11(L1_, 2), GBDE_O_ROW11(L1_, 3)};
#undef GBDE_O_ROW11
#define GBDE_O_ROW14(i) {L2_##i##_1, L2_##i##_2, L2_##i##_3, L2_##i##_4, L2_##i##_5, L2_##i##_6, \
                         L2_##i##_7, L2_##i##_8, L2_##i##_9, L2_##i##_10, L2_##i##_11,           \
                         L2_##i##_12, L2_##i##_13, L2_##i##_14}
    const double L2[4][14] = {GBDE_O_ROW14(1), GBDE_O_ROW14(2), GBDE_O_ROW14(3), GBDE_O_ROW14(4)};
#undef GBDE_O_ROW14
#define GBDE_O_D(j) {D##j##_1, D##j##_2, D##j##_3, D##j##_4, D##j##_5, D##j##_6, D##j##_7}
    const double D[18][7] = {GBDE_O_D(1),  GBDE_O_D(2),  GBDE_O_D(3),  GBDE_O_D(4),  GBDE_O_D(5),
                             GBDE_O_D(6),  GBDE_O_D(7),  GBDE_O_D(8),  GBDE_O_D(9),  GBDE_O_D(10),
                             GBDE_O_D(11), GBDE_O_D(12), GBDE_O_D(13), GBDE_O_D(14), GBDE_O_D(15),
                             GBDE_O_D(16), GBDE_O_D(17), GBDE_O_D(18)};
#undef GBDE_O_D
    double K[18][NMAX], y[NMAX];
    for (int j = 0; j < 11; ++j)
      for (int c = 0; c < n; ++c) K[j][c] = k[j][c];
    for (int i = 0; i < 3; ++i) {
      for (int c = 0; c < n; ++c) {
        double acc = 0.0;
        for (int j = 0; j < 11; ++j) acc += L1[i][j] * K[j][c];
        y[c] = u[c] + h * acc;
      }
      rhs(id, y, p, K[11 + i]);
    }
    for (int i = 0; i < 4; ++i) {
      for (int c = 0; c < n; ++c) {
        double acc = 0.0;
        for (int j = 0; j < 14; ++j) acc += L2[i][j] * K[j][c];
        y[c] = u[c] + h * acc;
      }
      rhs(id, y, p, K[14 + i]);
    }
    nf += 7;
    double w[18];
    for (int j = 0; j < 18; ++j) {
      double acc = 0.0;
      for (int m = 6; m >= 0; --m) acc = acc * th + D[j][m];
      w[j] = acc * th;
    }
    for (int c = 0; c < n; ++c) {
      double acc = 0.0;
      for (int j = 0; j < 18; ++j) acc += w[j] * K[j][c];
      out[c] = u[c] + h * acc;
    }
  }

  // ---- Rosenbrock23 (Shampine-Reichelt 1997)
  double ros23(double h, const Ctl& C, int& nf) {
    using gbde::tab::ros23::d;
    using gbde::tab::ros23::e32;
    if (!fresh) {
      jacobian(id, n, u, p, J);
      fresh = true;
    }
    LU W;
    W.n = n;
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) W.A[r * n + c] = (r == c ? 1.0 : 0.0) - h * d * J[r * n + c];
    W.factor();
    double y[NMAX], F1[NMAX], r3[NMAX], k3[NMAX], tmp[NMAX];
    W.solve(f0, k[0]);
    for (int c = 0; c < n; ++c) y[c] = u[c] + 0.5 * h * k[0][c];
    rhs(id, y, p, F1);
    for (int c = 0; c < n; ++c) tmp[c] = F1[c] - k[0][c];
    W.solve(tmp, k[1]);
    for (int c = 0; c < n; ++c) {
      k[1][c] += k[0][c];
      un[c] = u[c] + h * k[1][c];
    }
    rhs(id, un, p, k[2]);  // F2
    nf += 2;
    for (int c = 0; c < n; ++c)
      r3[c] = k[2][c] - e32 * (k[1][c] - F1[c]) - 2.0 * (k[0][c] - f0[c]);
    W.solve(r3, k3);
    double e[NMAX];
    for (int c = 0; c < n; ++c) e[c] = h / 6.0 * (k[0][c] - 2.0 * k[1][c] + k3[c]);
    return wrms(n, e, u, un, C.at, C.rt);
  }
  void ros23_interp(double th, double h, double* out) {
    using gbde::tab::ros23::d;
    const double w1 = th * (1.0 - th) / (1.0 - 2.0 * d), w2 = th * (th - 2.0 * d) / (1.0 - 2.0 * d);
    for (int c = 0; c < n; ++c) out[c] = u[c] + h * (w1 * k[0][c] + w2 * k[1][c]);
  }

  // ---- Rodas5 / Rodas5P (transformed form, Hairer-Wanner IV.7 (7.4')):
  //   (I/(h gamma) - J) u_i = f(y0 + sum_j a_ij u_j) + sum_j (C_ij / h) u_j
  //   a_7j = a_6j, a_76 = 1, a_8j = a_7j, a_87 = 1; y1 = U_8 + u_8; err = u_8.
  struct RodasTab {
    double g, a[8][7], C[8][7], H2[7], H3[7], H4[7];
  };
  static const RodasTab& rodas_tab(int which) {
    static RodasTab t5 = make_tab<5>(), t5p = make_tab<6>();
    return which == GBDE_ALG_RODAS5 ? t5 : t5p;
  }
  template <int W>
  static RodasTab make_tab() {
    RodasTab T{};
#define GBDE_FILL(NS, DNS)                                                                       \
    {                                                                                            \
      using namespace gbde::tab::NS;                                                             \
      T.g = gbde::tab::NS::gamma;                                                                \
      T.a[1][0] = a21;                                                                           \
      T.a[2][0] = a31; T.a[2][1] = a32;                                                          \
      T.a[3][0] = a41; T.a[3][1] = a42; T.a[3][2] = a43;                                         \
      T.a[4][0] = a51; T.a[4][1] = a52; T.a[4][2] = a53; T.a[4][3] = a54;                        \
      T.a[5][0] = a61; T.a[5][1] = a62; T.a[5][2] = a63; T.a[5][3] = a64; T.a[5][4] = a65;       \
      T.C[1][0] = C21;                                                                           \
      T.C[2][0] = C31; T.C[2][1] = C32;                                                          \
      T.C[3][0] = C41; T.C[3][1] = C42; T.C[3][2] = C43;                                         \
      T.C[4][0] = C51; T.C[4][1] = C52; T.C[4][2] = C53; T.C[4][3] = C54;                        \
      T.C[5][0] = C61; T.C[5][1] = C62; T.C[5][2] = C63; T.C[5][3] = C64; T.C[5][4] = C65;       \
      T.C[6][0] = C71; T.C[6][1] = C72; T.C[6][2] = C73; T.C[6][3] = C74; T.C[6][4] = C75;       \
      T.C[6][5] = C76;                                                                           \
      T.C[7][0] = C81; T.C[7][1] = C82; T.C[7][2] = C83; T.C[7][3] = C84; T.C[7][4] = C85;       \
      T.C[7][5] = C86; T.C[7][6] = C87;                                                          \
    }                                                                                            \
    {                                                                                            \
      using namespace gbde::tab::DNS;                                                            \
      const double h2[7] = {H2_1, H2_2, H2_3, H2_4, H2_5, H2_6, H2_7};                           \
      const double h3[7] = {H3_1, H3_2, H3_3, H3_4, H3_5, H3_6, H3_7};                           \
      const double h4[7] = {H4_1, H4_2, H4_3, H4_4, H4_5, H4_6, H4_7};                           \
      for (int j = 0; j < 7; ++j) { T.H2[j] = h2[j]; T.H3[j] = h3[j]; T.H4[j] = h4[j]; }         \
    }
    if (W == 5) {
      GBDE_FILL(rodas5, rodas5d)
    } else {
      GBDE_FILL(rodas5p, rodas5pd)
    }
#undef GBDE_FILL
    for (int j = 0; j < 5; ++j) T.a[6][j] = T.a[5][j];
    T.a[6][5] = 1.0;
    for (int j = 0; j < 6; ++j) T.a[7][j] = T.a[6][j];
    T.a[7][6] = 1.0;
    return T;
  }

  double rodas(double h, const Ctl& C, int& nf) {
    const RodasTab& T = rodas_tab(alg);
    if (!fresh) {
      rhs(id, u, p, f0);
      ++nf;
      jacobian(id, n, u, p, J);
      fresh = true;
    }
    LU W;
    W.n = n;
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c)
        W.A[r * n + c] = (r == c ? 1.0 / (h * T.g) : 0.0) - J[r * n + c];
    W.factor();
    double y[NMAX], fy[NMAX], rr[NMAX];
    W.solve(f0, k[0]);
    for (int s = 1; s < 8; ++s) {
      for (int c = 0; c < n; ++c) {
        double acc = u[c];
        for (int j = 0; j < s; ++j) acc += T.a[s][j] * k[j][c];
        y[c] = acc;
      }
      rhs(id, y, p, fy);
      for (int c = 0; c < n; ++c) {
        double acc = fy[c];
        for (int j = 0; j < s; ++j) acc += (T.C[s][j] / h) * k[j][c];
        rr[c] = acc;
      }
      W.solve(rr, k[s]);
    }
    nf += 7;
    for (int c = 0; c < n; ++c) un[c] = y[c] + k[7][c];
    return wrms(n, k[7], u, un, C.at, C.rt);
  }
  void rodas_interp(double th, double* out) {
    const RodasTab& T = rodas_tab(alg);
    for (int c = 0; c < n; ++c) {
      double k2 = 0, k3 = 0, k4 = 0;
      for (int j = 0; j < 7; ++j) {
        k2 += T.H2[j] * k[j][c];
        k3 += T.H3[j] * k[j][c];
        k4 += T.H4[j] * k[j][c];
      }
      out[c] = (1.0 - th) * u[c] + th * un[c] + th * (1.0 - th) * (k2 + th * (k3 + th * k4));
    }
  }

  // ||J||_inf (row sums of |J| in column order): the Rosenbrock methods'
  // stiffness estimate in a switching composite
  double jac_norm() const {
    double mx = 0.0;
    bool nan = false;
    for (int r = 0; r < n; ++r) {
      double s = 0.0;
      for (int c = 0; c < n; ++c) s += std::fabs(J[r * n + c]);
      nan |= s != s;
      mx = std::fmax(mx, s);
    }
    return nan ? NAN : mx;
  }
  double attempt(double h, const Ctl& C, int& nf) {
    switch (alg) {
      case GBDE_ALG_TSIT5: return tsit5(h, C, nf);
      case GBDE_ALG_VERN7: return vern7(h, C, nf);
      case GBDE_ALG_ROSENBROCK23: {
        const double E = ros23(h, C, nf);
        eig = jac_norm();
        return E;
      }
      default: {
        const double E = rodas(h, C, nf);
        eig = jac_norm();
        return E;
      }
    }
  }
  // Continue the trajectory at u with another method: f(u) carries over
  // (Rodas re-evaluates it after an accept, so it is evaluated here then);
  // Rodas gets its Jacobian at u now.
  void switch_to(int to, int& nf) {
    if ((alg == GBDE_ALG_RODAS5 || alg == GBDE_ALG_RODAS5P) && !fresh) {
      rhs(id, u, p, f0);
      ++nf;
    }
    alg = to;
    have11 = false;
    if (to == GBDE_ALG_RODAS5 || to == GBDE_ALG_RODAS5P) {
      jacobian(id, n, u, p, J);
      fresh = true;
    } else {
      fresh = false;
    }
  }
  void interp(double th, double h, double* out, int& nf) {
    switch (alg) {
      case GBDE_ALG_TSIT5: tsit5_interp(th, h, out); break;
      case GBDE_ALG_VERN7: vern7_interp(th, h, out, nf); break;
      case GBDE_ALG_ROSENBROCK23: ros23_interp(th, h, out); break;
      default: rodas_interp(th, out); break;
    }
  }
  void accept(int& nf) {
    for (int c = 0; c < n; ++c) u[c] = un[c];
    if (alg == GBDE_ALG_TSIT5) {
      for (int c = 0; c < n; ++c) f0[c] = k[6][c];
    } else if (alg == GBDE_ALG_VERN7) {
      if (have11) for (int c = 0; c < n; ++c) f0[c] = k[10][c];
      else { rhs(id, u, p, f0); ++nf; }
      have11 = false;
    } else if (alg == GBDE_ALG_ROSENBROCK23) {
      for (int c = 0; c < n; ++c) f0[c] = k[2][c];
      fresh = false;
    } else {
      fresh = false;
    }
  }
  int order() const {
    switch (alg) {
      case GBDE_ALG_TSIT5: return 5;
      case GBDE_ALG_VERN7: return 7;
      case GBDE_ALG_ROSENBROCK23: return 2;
      default: return 4;
    }
  }
};


// ------------------------------------------------------------ ODE driver
// One trajectory: PI controller (HNW I, II.4; Gustafsson), scaled RMS norm,
// HNW starting step, dense output at save times, tf snapping, return codes.
// stiff_alg != 0: the AutoTsit5(stiff_alg) composite (AutoSwitch with its
// published defaults: before every attempt after the first, stiffness =
// |eig dt / 3.5068| > 9/10 counts; > 10 successive stiff estimates switch
// Tsit5 to stiff_alg with dt * 2, > 3 successive non-stiff ones switch back
// with dt / 2; the stiff method steps with the controller constants Cs).
void solve_ode_traj(const Model& m, int alg, const Ctl& C, Out& o, int stiff_alg = 0,
                    const Ctl* Cs = nullptr) {
  const gbde_problem* P = o.P;
  const int64_t i = o.i;
  const int n = m.n;
  const double* p = P->p + (size_t)i * m.np;
  const double* u0 = P->u0 + (size_t)i * n;
  double t = P->t0[i];
  const double tf = P->tf[i];
  int js = 0, nacc = 0, nrej = 0, nf = 0;
  int64_t iters = 0;
  int ret = GBDE_RET_DEFAULT;
  while (js < P->n_save && o.ts(js) <= t) o.save(js++, u0, n);
  bool bad = !(tf >= t) || !std::isfinite(t) || !std::isfinite(tf);
  for (int c = 0; c < n; ++c) bad |= !std::isfinite(u0[c]);
  Stepper S;
  S.alg = stiff_alg ? GBDE_ALG_TSIT5 : alg;
  S.n = n;
  S.id = m.id;
  S.p = p;
  bool stiff = false;
  int count = 0;
  double dt = 0.0;
  CtlMem cm = ctl_start(C);
  if (bad) {
    ret = GBDE_RET_INITIALFAILURE;
  } else {
    S.init(u0, nf);
    if (C.dt0 > 0.0 || !C.adaptive) dt = C.dt0;
    else dt = init_dt(m, S.u, S.f0, p, tf - t, S.order(), C.at, C.rt, nf);
    if (C.dtmax > 0.0) dt = std::fmin(dt, C.dtmax);
    if (!(t < tf)) ret = GBDE_RET_SUCCESS;
    else if (!(dt > 0.0)) ret = GBDE_RET_DTLESSTHANMIN;
  }
  while (ret == GBDE_RET_DEFAULT) {
    if (stiff_alg && iters > 0) {
      const double stiffness = std::fabs(S.eig * dt / 3.5068);
      const bool s = stiffness > 0.9;  // NaN: not stiff
      count = s ? (count < 0 ? 1 : count + 1) : (count > 0 ? -1 : count - 1);
      if (!stiff && count > 10) {
        S.switch_to(stiff_alg, nf);
        stiff = true;
        dt = dt * 2.0;
      } else if (stiff && count < -3) {
        S.switch_to(GBDE_ALG_TSIT5, nf);
        stiff = false;
        dt = dt / 2.0;
      }
      if (C.dtmax > 0.0) dt = std::fmin(dt, C.dtmax);
    }
    const Ctl& Cc = stiff ? *Cs : C;
    const double rem = tf - t;
    double h = dt;
    bool last = false;
    if (h * (1.0 + 1e-10) >= rem) {
      h = rem;
      last = true;
    }
    const double E = S.attempt(h, C, nf);  // EEst^2
    ++iters;
    if (!C.adaptive || E <= 1.0) {
      double dtnew = h;
      if (C.adaptive) dtnew = h * ctl_accept_r(Cc, E, cm);
      const double tnew = last ? tf : t + h;
      while (js < P->n_save) {
        const double ts = o.ts(js);
        if (!(ts <= tnew)) break;
        if (ts >= tnew) {
          o.save(js, S.un, n);
        } else {
          double tmp[NMAX];
          S.interp((ts - t) / h, h, tmp, nf);
          o.save(js, tmp, n);
        }
        ++js;
      }
      S.accept(nf);
      t = tnew;
      ++nacc;
      bool fin = true;
      for (int c = 0; c < n; ++c) fin &= std::isfinite(S.u[c]);
      if (!fin) ret = GBDE_RET_UNSTABLE;
      else if (last) ret = GBDE_RET_SUCCESS;
      dt = C.dtmax > 0.0 ? std::fmin(dtnew, C.dtmax) : dtnew;
    } else {
      ++nrej;
      dt = h * ctl_reject_r(Cc, E);
    }
    if (ret == GBDE_RET_DEFAULT) {
      if (iters >= C.maxiters) ret = GBDE_RET_MAXITERS;
      else if (C.adaptive && (dt < C.dtmin || dt <= 4.0 * 2.220446049250313e-16 * std::fabs(t)))
        ret = GBDE_RET_DTLESSTHANMIN;
    }
  }
  double nanv[NMAX];
  for (int c = 0; c < n; ++c) nanv[c] = NAN;
  for (; js < P->n_save; ++js) o.save(js, nanv, n);
  gbde_outputs* O = o.O;
  O->retcode[i] = ret;
  if (O->naccept) O->naccept[i] = nacc;
  if (O->nreject) O->nreject[i] = nrej;
  if (O->nf) O->nf[i] = nf;
  if (O->t_end) O->t_end[i] = t;
  if (O->method) O->method[i] = S.alg;
}

// ------------------------------------------------- Philox4x32-10 + normals
// Salmon et al., SC'11.  Counter (block_lo, block_hi, traj_lo, traj_hi), key
// (seed_lo, seed_hi).  Box-Muller with series log / sin / cos evaluated with
// explicit fma (compiled with -ffp-contract=off so no other contraction).
void philox(const uint32_t in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

template <class T> T fma_t(T a, T b, T c);
template <> double fma_t(double a, double b, double c) { return std::fma(a, b, c); }
template <> float fma_t(float a, float b, float c) { return std::fmaf(a, b, c); }

// log x = e ln2 + 2 atanh((m-1)/(m+1)), m in [1/sqrt2, sqrt2)
template <class T>
T series_log(T x, int nterms, T ln2hi, T ln2lo, T sqrth) {
  int e;
  T m = std::frexp(x, &e);
  if (m < sqrth) { m = m + m; e -= 1; }
  const T s = (m - T(1)) / (m + T(1));
  const T s2 = s * s;
  T acc = T(1) / T(2 * nterms + 1);
  for (int k = nterms - 1; k >= 0; --k) acc = fma_t<T>(acc, s2, T(1) / T(2 * k + 1));
  const T lm = (s + s) * acc;
  const T fe = (T)e;
  return fma_t<T>(fe, ln2hi, lm) + fe * ln2lo;
}

template <class T>
void series_sincos2pi(T u, int nterms, T pio2hi, T pio2lo, T& co, T& si) {
  const T v = u * T(4);
  const T qf = std::floor(v);
  T f = v - qf;
  int q = (int)qf;
  if (f > T(0.5)) { f = f - T(1); q += 1; }
  q &= 3;
  const T r = fma_t<T>(f, pio2hi, f * pio2lo);
  const T r2 = r * r;
  std::vector<T> sc(nterms + 1), cc(nterms + 1);
  T fs = 1, fc = 1;
  for (int k = 0; k <= nterms; ++k) {
    sc[k] = ((k & 1) ? T(-1) : T(1)) / fs;
    cc[k] = ((k & 1) ? T(-1) : T(1)) / fc;
    fs = fs * T((2 * k + 2) * (2 * k + 3));
    fc = fc * T((2 * k + 1) * (2 * k + 2));
  }
  T sp = sc[nterms], cp = cc[nterms];
  for (int k = nterms - 1; k >= 0; --k) {
    sp = fma_t<T>(sp, r2, sc[k]);
    cp = fma_t<T>(cp, r2, cc[k]);
  }
  const T sr = r * sp, cr = cp;
  switch (q) {
    case 0: co = cr; si = sr; break;
    case 1: co = -sr; si = cr; break;
    case 2: co = -cr; si = -sr; break;
    default: co = sr; si = -cr; break;
  }
}

void normal_pair_f64(uint64_t seed, uint64_t traj, uint64_t b, double& z0, double& z1) {
  const uint32_t ctr[4] = {(uint32_t)b, (uint32_t)(b >> 32), (uint32_t)traj, (uint32_t)(traj >> 32)};
  uint32_t r[4];
  philox(ctr, (uint32_t)seed, (uint32_t)(seed >> 32), r);
  const uint64_t a = ((uint64_t)(r[0] >> 5) << 26) | (r[1] >> 6);
  const uint64_t c = ((uint64_t)(r[2] >> 5) << 26) | (r[3] >> 6);
  const double u1 = ((double)a + 0.5) * 0x1p-53, u2 = (double)c * 0x1p-53;
  const double rad = std::sqrt(-2.0 * series_log<double>(u1, 12, 0.6931471805599453,
                                                          2.3190468138462996e-17,
                                                          0.7071067811865476));
  double co, si;
  series_sincos2pi<double>(u2, 9, 1.5707963267948966, 6.123233995736766e-17, co, si);
  z0 = rad * co;
  z1 = rad * si;
}

void normal_quad_f32(uint64_t seed, uint64_t traj, uint64_t b, float* z) {
  const uint32_t ctr[4] = {(uint32_t)b, (uint32_t)(b >> 32), (uint32_t)traj, (uint32_t)(traj >> 32)};
  uint32_t r[4];
  philox(ctr, (uint32_t)seed, (uint32_t)(seed >> 32), r);
  float u[4];
  for (int k = 0; k < 4; ++k) u[k] = (float)(r[k] >> 8) * 0x1p-24f;
  u[0] = ((float)(r[0] >> 8) + 0.5f) * 0x1p-24f;
  u[2] = ((float)(r[2] >> 8) + 0.5f) * 0x1p-24f;
  for (int k = 0; k < 2; ++k) {
    const float rad = std::sqrt(-2.0f * series_log<float>(u[2 * k], 6, 0.693147182f,
                                                           -1.90465421e-09f, 0.707106781f));
    float co, si;
    series_sincos2pi<float>(u[2 * k + 1], 5, 1.57079637f, -4.37113883e-08f, co, si);
    z[2 * k] = rad * co;
    z[2 * k + 1] = rad * si;
  }
}

// Per-trajectory normal stream; f32 = 1 reads the FP32 stream (promoted).
struct Normals {
  uint64_t seed, traj, d = 0, blk = ~0ull;
  int f32;
  double buf[4];
  double next() {
    const int per = f32 ? 4 : 2;
    const uint64_t b = d / per;
    if (b != blk) {
      if (f32) {
        float z[4];
        normal_quad_f32(seed, traj, b, z);
        for (int k = 0; k < 4; ++k) buf[k] = z[k];
      } else {
        normal_pair_f64(seed, traj, b, buf[0], buf[1]);
      }
      blk = b;
    }
    return buf[d++ % per];
  }
};

// ------------------------------------------------------------ SDE drivers
void finish(Out& o, int n, int js, int ret, int nacc, int nrej, int nf, double t, int alg) {
  double nanv[NMAX];
  for (int c = 0; c < n; ++c) nanv[c] = NAN;
  for (; js < o.P->n_save; ++js) o.save(js, nanv, n);
  gbde_outputs* O = o.O;
  O->retcode[o.i] = ret;
  if (O->naccept) O->naccept[o.i] = nacc;
  if (O->nreject) O->nreject[o.i] = nrej;
  if (O->nf) O->nf[o.i] = nf;
  if (O->t_end) O->t_end[o.i] = t;
  if (O->method) O->method[o.i] = alg;
}

// Euler-Maruyama (Kloeden-Platen): step n spans [t0 + n h, min(t0 + (n+1) h, tf)],
// normal n*N + c drives component c; linear interpolation at save times.
void solve_em_traj(const Model& m, const Ctl& C, uint64_t seed, int f32, Out& o) {
  const gbde_problem* P = o.P;
  const int64_t i = o.i;
  const int n = m.n;
  const double* p = P->p + (size_t)i * m.np;
  double u[NMAX];
  for (int c = 0; c < n; ++c) u[c] = P->u0[(size_t)i * n + c];
  const double t0 = P->t0[i], tf = P->tf[i], h = C.dt0;
  int js = 0;
  while (js < P->n_save && o.ts(js) <= t0) o.save(js++, u, n);
  bool bad = !(tf >= t0) || !std::isfinite(t0) || !std::isfinite(tf);
  for (int c = 0; c < n; ++c) bad |= !std::isfinite(u[c]);
  if (bad) return finish(o, n, js, GBDE_RET_INITIALFAILURE, 0, 0, 0, t0, GBDE_ALG_EM);
  Normals z{seed, (uint64_t)i};
  z.f32 = f32;
  int ret = GBDE_RET_SUCCESS;
  int64_t k = 0;
  double t = t0;
  while (t < tf) {
    if (k >= C.maxiters) { ret = GBDE_RET_MAXITERS; break; }
    double tn1 = t0 + (double)(k + 1) * h;
    if (tn1 * (1.0 + 1e-14) >= tf || tn1 > tf) tn1 = tf;
    const double hs = tn1 - t, sq = std::sqrt(hs);
    double fu[NMAX], gu[NMAX], un[NMAX];
    rhs(m.id, u, p, fu);
    noise(m.id, u, p, gu);
    for (int c = 0; c < n; ++c) un[c] = u[c] + fu[c] * hs + gu[c] * (sq * z.next());
    while (js < P->n_save) {
      const double ts = o.ts(js);
      if (!(ts <= tn1)) break;
      if (ts >= tn1) o.save(js, un, n);
      else {
        const double th = (ts - t) / hs;
        double tmp[NMAX];
        for (int c = 0; c < n; ++c) tmp[c] = u[c] + th * (un[c] - u[c]);
        o.save(js, tmp, n);
      }
      ++js;
    }
    bool fin = true;
    for (int c = 0; c < n; ++c) { u[c] = un[c]; fin &= std::isfinite(un[c]); }
    t = tn1;
    ++k;
    if (!fin) { ret = GBDE_RET_UNSTABLE; break; }
  }
  finish(o, n, js, ret, (int)k, 0, (int)(2 * k), t, GBDE_ALG_EM);
}

// SRIW1 (Roessler 2010) with rejection sampling with memory (Rackauckas &
// Nie 2017): future Brownian pieces on a stack (nearest on top), split by a
// Brownian bridge when longer than needed; 8 entries, the two farthest
// pieces merge when full.
struct Piece {
  double dt, W[NMAX], Z[NMAX];
};

// One trajectory of a 4-stage SRI (Roessler's form; Tab = SosriTab or
// Sriw1Tab, tableaus.h):
//   H0_i = X + sum_j A0_ij f(H0_j) h + sum_j B0_ij g(H1_j) I10/h
//   H1_i = X + sum_j A1_ij f(H0_j) h + sum_j B1_ij g(H1_j) sqrt(h)
//   X'   = X + h sum_i al_i f(H0_i)
//            + sum_i (b1_i dW + b2_i I11/sqrt(h) + b3_i I10/h + b4_i I111/h) g(H1_i)
// Error estimate (Rackauckas & Nie, DCDS-B 22 (2017)): the embedded Euler
// drift and the terms of strong order 1.5,
//   E = h |sum_i al_i f(H0_i) - f(X)| + |sum_i (b3_i I10/h + b4_i I111/h) g(H1_i)|.
template <class Tab>
void solve_sri_traj(const Model& m, const Ctl& C, uint64_t seed, int f32, Out& o, int alg) {
  const gbde_problem* P = o.P;
  const int64_t i = o.i;
  const int n = m.n;
  const double* p = P->p + (size_t)i * m.np;
  double u[NMAX];
  for (int c = 0; c < n; ++c) u[c] = P->u0[(size_t)i * n + c];
  const double t0 = P->t0[i], tf = P->tf[i];
  int js = 0;
  while (js < P->n_save && o.ts(js) <= t0) o.save(js++, u, n);
  bool bad = !(tf >= t0) || !std::isfinite(t0) || !std::isfinite(tf);
  for (int c = 0; c < n; ++c) bad |= !std::isfinite(u[c]);
  if (bad) return finish(o, n, js, GBDE_RET_INITIALFAILURE, 0, 0, 0, t0, alg);
  Normals z{seed, (uint64_t)i};
  z.f32 = f32;
  Piece stk[8];
  int sp = 0;
  int nf = 0, nacc = 0, nrej = 0;
  double t = t0, h;
  if (C.dt0 > 0.0) h = C.dt0;
  else {
    double f0[NMAX];
    rhs(m.id, u, p, f0);
    ++nf;
    h = init_dt(m, u, f0, p, tf - t0, 1, C.at, C.rt, nf);
  }
  if (C.dtmax > 0.0) h = std::fmin(h, C.dtmax);
  int ret = t < tf ? GBDE_RET_DEFAULT : GBDE_RET_SUCCESS;
  int64_t iters = 0;
  CtlMem cm = ctl_start(C);
  while (ret == GBDE_RET_DEFAULT) {
    const double rem = tf - t;
    double hs = h;
    bool last = false;
    if (hs * (1.0 + 1e-10) >= rem) { hs = rem; last = true; }
    // increments over [t, t + hs]
    double dW[NMAX] = {0}, dZ[NMAX] = {0}, acc = 0.0;
    while (true) {
      const double r = hs - acc;
      if (!(r > 1e-14 * hs)) break;
      if (sp > 0) {
        Piece& top = stk[sp - 1];
        if (top.dt <= r * (1.0 + 1e-12)) {
          acc += top.dt;
          for (int c = 0; c < n; ++c) { dW[c] += top.W[c]; dZ[c] += top.Z[c]; }
          --sp;
        } else {
          const double frac = r / top.dt, sd = std::sqrt(r * (top.dt - r) / top.dt);
          for (int c = 0; c < n; ++c) {
            const double wr = top.W[c] * frac + sd * z.next();
            const double zr = top.Z[c] * frac + sd * z.next();
            dW[c] += wr; dZ[c] += zr;
            top.W[c] -= wr; top.Z[c] -= zr;
          }
          top.dt -= r;
          acc = hs;
        }
      } else {
        const double sq = std::sqrt(r);
        for (int c = 0; c < n; ++c) {
          dW[c] += sq * z.next();
          dZ[c] += sq * z.next();
        }
        acc = hs;
      }
    }
    const double sqh = std::sqrt(hs), ih = 1.0 / hs, isqh = 1.0 / std::sqrt(hs);
    double I10[NMAX], I11[NMAX], I111[NMAX];
    for (int c = 0; c < n; ++c) {
      I10[c] = 0.5 * hs * (dW[c] + dZ[c] * 0.57735026918962576451);
      I11[c] = 0.5 * (dW[c] * dW[c] - hs);
      I111[c] = (dW[c] * dW[c] * dW[c] - 3.0 * hs * dW[c]) * (1.0 / 6.0);
    }
    // stage values: f at H0_i, g at H1_i, in stage order; a stage whose H0
    // (H1) row is empty sits at X
    double F[4][NMAX], G[4][NMAX], Y[NMAX], un[NMAX], err[NMAX];
    rhs(m.id, u, p, F[0]);
    noise(m.id, u, p, G[0]);
    int nfs = 1;
    for (int s = 1; s < 4; ++s) {
      bool h0x = true, h1x = true;
      for (int j = 0; j < s; ++j) {
        h0x = h0x && Tab::A0[s][j] == 0.0 && Tab::B0[s][j] == 0.0;
        h1x = h1x && Tab::A1[s][j] == 0.0 && Tab::B1[s][j] == 0.0;
      }
      if (h0x) {
        for (int c = 0; c < n; ++c) F[s][c] = F[0][c];
      } else {
        for (int c = 0; c < n; ++c) {
          double af = 0.0, bg = 0.0;
          for (int j = 0; j < s; ++j) {
            af += Tab::A0[s][j] * F[j][c];
            bg += Tab::B0[s][j] * G[j][c];
          }
          Y[c] = u[c] + af * hs + bg * I10[c] * ih;
        }
        rhs(m.id, Y, p, F[s]);
        // counted when the method uses it (alpha or a later A0 / A1 column)
        bool used = Tab::al[s] != 0.0;
        for (int k = s + 1; k < 4; ++k) used = used || Tab::A0[k][s] != 0.0 || Tab::A1[k][s] != 0.0;
        nfs += used ? 1 : 0;
      }
      if (h1x) {
        for (int c = 0; c < n; ++c) G[s][c] = G[0][c];
      } else {
        for (int c = 0; c < n; ++c) {
          double af = 0.0, bg = 0.0;
          for (int j = 0; j < s; ++j) {
            af += Tab::A1[s][j] * F[j][c];
            bg += Tab::B1[s][j] * G[j][c];
          }
          Y[c] = u[c] + af * hs + bg * sqh;
        }
        noise(m.id, Y, p, G[s]);
      }
    }
    nf += nfs;
    for (int c = 0; c < n; ++c) {
      double drift = 0.0, sto = 0.0, en3 = 0.0, en4 = 0.0, ed = 0.0;
      for (int s = 0; s < 4; ++s) {
        drift += Tab::al[s] * F[s][c];
        ed += (Tab::al[s] - (s == 0 ? 1.0 : 0.0)) * F[s][c];
        sto += (Tab::b[0][s] * dW[c] + Tab::b[1][s] * I11[c] * isqh + Tab::b[2][s] * I10[c] * ih +
                Tab::b[3][s] * I111[c] * ih) * G[s][c];
        en3 += Tab::b[2][s] * G[s][c];
        en4 += Tab::b[3][s] * G[s][c];
      }
      un[c] = u[c] + hs * drift + sto;
      const double en = en3 * I10[c] * ih + en4 * I111[c] * ih;
      err[c] = std::fabs(hs * ed) + std::fabs(en);
    }
    const double E = wrms(n, err, u, un, C.at, C.rt);
    ++iters;
    if (!C.adaptive || E <= 1.0) {
      const double tnew = last ? tf : t + hs;
      while (js < P->n_save) {
        const double ts = o.ts(js);
        if (!(ts <= tnew)) break;
        if (ts >= tnew) o.save(js, un, n);
        else {
          const double th = (ts - t) / hs;
          double tmp[NMAX];
          for (int c = 0; c < n; ++c) tmp[c] = u[c] + th * (un[c] - u[c]);
          o.save(js, tmp, n);
        }
        ++js;
      }
      bool fin = true;
      for (int c = 0; c < n; ++c) { u[c] = un[c]; fin &= std::isfinite(un[c]); }
      t = tnew;
      ++nacc;
      if (!fin) ret = GBDE_RET_UNSTABLE;
      else if (last) ret = GBDE_RET_SUCCESS;
      if (C.adaptive) h = hs * ctl_accept_r(C, E, cm);
    } else {
      ++nrej;
      if (sp == 8) {  // merge the two farthest pieces
        stk[0].dt += stk[1].dt;
        for (int c = 0; c < n; ++c) { stk[0].W[c] += stk[1].W[c]; stk[0].Z[c] += stk[1].Z[c]; }
        for (int k = 1; k < 7; ++k) stk[k] = stk[k + 1];
        sp = 7;
      }
      stk[sp].dt = hs;
      for (int c = 0; c < n; ++c) { stk[sp].W[c] = dW[c]; stk[sp].Z[c] = dZ[c]; }
      ++sp;
      h = hs * ctl_reject_r(C, E);
    }
    if (C.dtmax > 0.0) h = std::fmin(h, C.dtmax);
    if (ret == GBDE_RET_DEFAULT) {
      if (iters >= C.maxiters) ret = GBDE_RET_MAXITERS;
      else if (C.adaptive && (h < C.dtmin || h <= 4.0 * 2.220446049250313e-16 * std::fabs(t)))
        ret = GBDE_RET_DTLESSTHANMIN;
    }
  }
  finish(o, n, js, ret, nacc, nrej, nf, t, alg);
}

}  // namespace

// ------------------------------------------------------------- C entry
extern "C" {

// Solve the ensemble on the CPU in FP64 with `nthreads` std::threads
// (EnsembleThreads-equivalent; nthreads <= 1 runs serially, EnsembleSerial).
// Same structs as gbde_ensemble_solve; host pointers only.  noise_f32 = 1
// drives the SDE methods with the FP32 normal stream (promoted to FP64), the
// stream the mixed-precision GPU path draws.
int oracle_ensemble_solve(const gbde_problem* P, const gbde_opts* O, gbde_outputs* out,
                          int nthreads, int noise_f32) {
  Model m;
  if (!P || !O || !out || !model_of(P->model, m)) return GBDE_ERR_INVALID;
  if (P->n_state != m.n || P->n_param != m.np || P->mem != GBDE_MEM_HOST) return GBDE_ERR_INVALID;
  Ctl C{O->abstol, O->reltol, O->qmin, O->qmax, O->gamma, O->beta1, O->beta2, O->qsteady_min,
        O->qsteady_max, O->qoldinit, O->dtmin, O->dtmax, O->dt, O->maxiters, O->adaptive,
        gbde::ctl_consts(O->beta1, O->beta2, O->gamma, O->qmin, O->qmax, O->qsteady_min,
                         O->qsteady_max, O->qoldinit)};
  const int alg = O->alg;
  // AutoTsit5 composites: the stiff method and its own PI exponents (its
  // option defaults: Rosenbrock23 1/3, 0; Rodas5 1/5, 0)
  const int stiff_alg = alg == GBDE_ALG_AUTOTSIT5_ROSENBROCK23 ? GBDE_ALG_ROSENBROCK23
                        : alg == GBDE_ALG_AUTOTSIT5_RODAS5     ? GBDE_ALG_RODAS5
                                                               : 0;
  Ctl Cs = C;
  if (stiff_alg) {
    Cs.beta1 = stiff_alg == GBDE_ALG_ROSENBROCK23 ? 1.0 / 3.0 : 1.0 / 5.0;
    Cs.beta2 = 0.0;
    Cs.k = gbde::ctl_consts(Cs.beta1, Cs.beta2, O->gamma, O->qmin, O->qmax, O->qsteady_min,
                            O->qsteady_max, O->qoldinit);
  }
  const int64_t N = P->n_traj;
  std::atomic<int64_t> next{0};
  auto work = [&]() {
    const int64_t chunk = 64;
    while (true) {
      const int64_t b = next.fetch_add(chunk);
      if (b >= N) break;
      const int64_t e = b + chunk < N ? b + chunk : N;
      for (int64_t i = b; i < e; ++i) {
        Out o{P, out, i};
        if (alg == GBDE_ALG_EM) solve_em_traj(m, C, O->seed, noise_f32, o);
        else if (alg == GBDE_ALG_SOSRI)
          solve_sri_traj<gbde::tab::SosriTab>(m, C, O->seed, noise_f32, o, alg);
        else if (alg == GBDE_ALG_SRIW1)
          solve_sri_traj<gbde::tab::Sriw1Tab>(m, C, O->seed, noise_f32, o, alg);
        else if (stiff_alg) solve_ode_traj(m, alg, C, o, stiff_alg, &Cs);
        else solve_ode_traj(m, alg, C, o);
      }
    }
  };
  if (nthreads <= 1) {
    work();
  } else {
    std::vector<std::thread> pool;
    for (int k = 0; k < nthreads; ++k) pool.emplace_back(work);
    for (auto& th : pool) th.join();
  }
  return GBDE_OK;
}

void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  philox(ctr, key[0], key[1], out);
}

void oracle_normals(uint64_t seed, uint64_t traj, uint64_t counter, int64_t n, int f32,
                    double* out) {
  Normals z{seed, traj};
  z.f32 = f32;
  z.d = counter;
  for (int64_t k = 0; k < n; ++k) out[k] = z.next();
}

// x = A^{-1} b by the oracle's partial-pivot LU (A row-major n x n, n <= 16):
// the linear solve of its Rosenbrock steppers, exposed for its own tests.
int oracle_lu_solve(int n, const double* A, const double* b, double* x) {
  if (n < 1 || n > NMAX) return GBDE_ERR_INVALID;
  LU W;
  W.n = n;
  for (int k = 0; k < n * n; ++k) W.A[k] = A[k];
  W.factor();
  W.solve(b, x);
  return GBDE_OK;
}

// Controller arithmetic of later solves: 0 = the kernels' FP32 series
// (controller.h, identical steps), 1 = FP64 pow() (see g_ctl_pow64).
void oracle_set_controller(int mode) { g_ctl_pow64 = mode == 1; }

// Mismatches between the controller's exact helpers (controller.h: ctl_frexp,
// ctl_i2f, the rint and ldexp steps of ctl_exp2f) and the C library's frexpf,
// (float), rintf and ldexpf, over the ranges the controller feeds them: every
// 97th positive normal float, every |i| <= 200, and y in [-60, 60] by 1/64
// (the rounding ties at k + 1/2 included).
int64_t oracle_ctl_selfcheck() {
  int64_t bad = 0;
  for (uint32_t b = 0x00800000u; b < 0x7f800000u; b += 97u) {
    float x;
    memcpy(&x, &b, sizeof(x));
    int e0 = 0, e1 = 0;
    const float m0 = frexpf(x, &e0), m1 = gbde::ctl_frexp(x, e1);
    bad += (m0 != m1 || e0 != e1);
  }
  for (int i = -200; i <= 200; ++i) bad += ((float)i != gbde::ctl_i2f(i));
  for (int j = -60 * 64; j <= 60 * 64; ++j) {
    const float y = (float)j / 64.0f;
    const float r = y + gbde::kCtlRound;
    uint32_t rb;
    memcpy(&rb, &r, sizeof(rb));
    const int ki = (int)(rb - 0x4b400000u);
    const float k = r - gbde::kCtlRound;
    bad += (k != rintf(y) || (float)ki != k);
    const float scaled = 1.25f * gbde::ctl_bitsf((uint32_t)(127 + ki) << 23);
    bad += (scaled != ldexpf(1.25f, ki));
  }
  return bad;
}

// The controller's integer-pipe double -> float rounding (d2f_rn_bits,
// common.cuh), for its test against the hardware conversion.
void oracle_d2f_rn(const double* x, float* out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) out[i] = gbde::d2f_rn_bits(x[i]);
}

int oracle_hardware_threads(void) {
  const unsigned h = std::thread::hardware_concurrency();
  return h ? (int)h : 1;
}

}  // extern "C"
