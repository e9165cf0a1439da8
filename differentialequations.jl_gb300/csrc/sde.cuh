// sde.cuh -- Euler-Maruyama and adaptive SRI (strong order 1.5) ensemble
// drivers with diagonal noise, driven by the Philox normal stream.
//
// The reference re-exports SDEProblem / SDEFunction (test/qa/qa.jl:102-103);
// its EM and SOSRI solvers live in StochasticDiffEq, which the reference does
// not depend on (Project.toml:6-10).  Methods restated here:
//  * EM: u_{n+1} = u_n + f(u_n) h + g(u_n) dW_n, dW_n = sqrt(h) z (Kloeden &
//    Platen 1992).  Save times are linearly interpolated between steps.
//  * SRI: A. Roessler, "Runge-Kutta methods for the strong approximation of
//    solutions of stochastic differential equations", SIAM J. Numer. Anal.
//    48 (2010) 922-952, the SRIW1 tableau (4 stages, strong order 1.5 for
//    diagonal noise) with I_(1,0) = h/2 (dW + dZ/sqrt(3)), dZ an independent
//    Brownian increment.  Error estimate (Rackauckas & Nie, DCDS-B 22 (2017)):
//      E = delta*h*|sum_i (alpha_i - [i==1]) f(H0_i)|
//          + |sum_i (beta3_i I10/h + beta4_i I111/h) g(H1_i)|,  delta = 1.
//  * Rejection sampling with memory (same paper): a rejected step's Brownian
//    increments (dt, dW, dZ) are pushed onto a per-trajectory stack of future
//    pieces; the next attempt consumes pieces front to back and splits a piece
//    that is longer than needed with a Brownian bridge,
//      W_r ~ N(W_piece r/dt_piece, r (dt_piece - r)/dt_piece),
//    so the path stays one Brownian path whatever the accept/reject history.
//    Every normal comes from the counter-based stream in draw order, so the
//    host can replay a trajectory exactly.
#pragma once
#include "philox.h"
#include "solver.cuh"
#include "tableaus.h"

namespace gbde {


// Reader of one trajectory's normal stream: draw d is normal d % PER of
// Philox block d / PER (PER = 4 FP32 or 2 FP64 normals per block).  The
// unused normals of the current block sit in registers with the next one
// first and shift down on each draw, so no run-time index puts them in local
// memory.
template <class T>
struct NormalStream {
  uint64_t seed, traj, blk;  // blk: the next block to generate
  T z0, z1, z2, z3;
  int left;                  // unused normals of the current block
  GBDE_D void init(uint64_t s, uint64_t tr) {
    seed = s;
    traj = tr;
    blk = 0;
    left = 0;
  }
  GBDE_D T next() {
    if (left == 0) {
      if constexpr (sizeof(T) == 8) {
        double a, b;
        philox_normal_pair_f64(seed, traj, blk, a, b);
        z0 = (T)a;
        z1 = (T)b;
        z2 = z3 = T(0);
        left = 2;
      } else {
        float q[4];
        philox_normal_quad_f32(seed, traj, blk, q);
        z0 = q[0];
        z1 = q[1];
        z2 = q[2];
        z3 = q[3];
        left = 4;
      }
      ++blk;
    }
    const T z = z0;
    z0 = z1;
    z1 = z2;
    z2 = z3;
    --left;
    return z;
  }
};

template <int N, class T>
GBDE_D void finish_sde(const KArgs& a, int64_t i, int ret, int js, int nacc, int nrej, int nfev,
                       double t, int alg, double dt1) {
  if (js < a.n_save) {
    T nanv[N];
#pragma unroll
    for (int c = 0; c < N; ++c) nanv[c] = (T)__longlong_as_double(0x7ff8000000000000ll);
    for (; js < a.n_save; ++js) store_state<N>(a, i, js, nanv);
  }
  a.retcode[i] = ret;
  if (a.naccept) a.naccept[i] = nacc;
  if (a.nreject) a.nreject[i] = nrej;
  if (a.nf) a.nf[i] = nfev;
  if (a.t_end) a.t_end[i] = t;
  if (a.method_out) a.method_out[i] = alg;
  if (a.dt_first) a.dt_first[i] = dt1;
}

// ------------------------------------------------------------------ EM
// Step n covers [t0 + n h, min(t0 + (n+1) h, tf)]; the normal for
// component c of step n is draw n*N + c of the trajectory's stream.

// End of EM step n in FP64 (as the FP64 loop of em_all computes it): the
// step is the last one when this test holds.
GBDE_D bool em_last_step(double t0, double tf, double h, int64_t n) {
  const double tn1 = t0 + (double)(n + 1) * h;
  return tn1 * (1.0 + 1e-14) >= tf || tn1 > tf;
}

// The EM steps of one trajectory with FP32 state (GBDE_PREC_MIXED).  The loop
// runs on a step counter with no FP64 arithmetic: h and sqrt(h) are FP32
// constants for every step but the last, whose length tf - t_n is computed
// once, and the step in which each save point falls is found (a few FP64
// operations per save point) before the loop reaches it.  The FP64 loop spends
// ~20 FP64-pipe instructions per step on the same bookkeeping, which bounds it
// on GB300's narrow FP64 pipe; this one is bound by the normal stream (Philox on
// the integer pipe, Box-Muller on the MUFU pipe).  Step boundaries are the FP64
// loop's t0 + n h: a step's length differs from h only by the rounding of
// those boundaries, below FP32 resolution.
template <class M>
__device__ void em_steps_f32(const KArgs& a, int64_t i, double t0, double tf, double h, float* u,
                             const float* p, int js, NormalStream<float>& ns, uint64_t t_start) {
  constexpr int N = M::N;
  constexpr int64_t kNever = 0x7fffffffffffffffll;
  // index of the last step (-1: no step)
  int64_t nl = -1;
  if (t0 < tf) {
    const double m = (tf - t0) / h;
    if (!(m <= (double)a.maxiters + 2.0)) {
      nl = kNever - 1;  // more steps than maxiters: the loop stops at maxiters
    } else {
      nl = m > 1.0 ? (int64_t)m - 1 : 0;
      for (int it = 0; it < 8 && nl > 0 && em_last_step(t0, tf, h, nl - 1); ++it) --nl;
      for (int it = 0; it < 8 && !em_last_step(t0, tf, h, nl); ++it) ++nl;
    }
  }
  const int64_t nrun = nl + 1 < a.maxiters ? nl + 1 : a.maxiters;
  // end of step n in FP64, and the step in which save point j falls
  auto t_end = [&](int64_t n) { return n >= nl ? tf : t0 + (double)(n + 1) * h; };
  auto save_step = [&](int j) -> int64_t {
    if (j >= a.n_save) return kNever;
    const double ts = save_time(a, i, j);
    if (!(ts <= tf) || nl < 0) return kNever;
    const double kd = (ts - t0) / h;
    int64_t k = kd < (double)nl ? (int64_t)kd - 1 : nl;
    k = k < 0 ? 0 : k;
    // the estimate is within a step or two; the bounds only matter where h is
    // below the FP64 resolution of t (the step boundaries then repeat)
    for (int it = 0; it < 64 && k > 0 && t_end(k - 1) >= ts; ++it) --k;
    for (int it = 0; it < 64 && k < nl && t_end(k) < ts; ++it) ++k;
    return k;
  };
  const float hT = (float)h, sq = (float)sqrt(h);
  float hTl = hT, sql = sq;
  if (nl >= 0 && nl < kNever - 1) {
    const double hl = tf - (nl > 0 ? t0 + (double)nl * h : t0);
    hTl = (float)hl;
    sql = (float)sqrt(hl);
  }
  int64_t ks = save_step(js);
  int ret = GBDE_RET_SUCCESS;
  int64_t n = 0;
  // register copies of the state and parameters (no pointer into the
  // caller's arrays inside the loop)
  float ur[N], pr[M::NP];
#pragma unroll
  for (int c = 0; c < N; ++c) ur[c] = u[c];
#pragma unroll
  for (int k = 0; k < M::NP; ++k) pr[k] = p[k];
  for (; n < nrun; ++n) {
    // the optional device deadline, every 1024 steps
    if (a.timeout_ns && (n & 1023) == 0 && n > 0 && global_ns() - t_start > a.timeout_ns) {
      ret = GBDE_RET_TIMEOUT;
      atomicOr(a.flag, 1);
      break;
    }
    const bool lastn = n == nl;
    const float hs = lastn ? hTl : hT, sh = lastn ? sql : sq;
    float fu[N], gu[N], un[N];
    M::f(fu, ur, pr);
    M::g(gu, ur, pr);
#pragma unroll
    for (int c = 0; c < N; ++c) un[c] = ur[c] + fu[c] * hs + gu[c] * (sh * ns.next());
    while (n == ks) {  // save points in (t_n, t_{n+1}]
      const double ts = save_time(a, i, js), tn1 = t_end(n);
      const double tn = n > 0 ? t0 + (double)n * h : t0;
      if (ts >= tn1) {
        store_state<N>(a, i, js, un);
      } else {
        const float th = (float)((ts - tn) / (tn1 - tn));
        float tmp[N];
#pragma unroll
        for (int c = 0; c < N; ++c) tmp[c] = ur[c] + th * (un[c] - ur[c]);
        store_state<N>(a, i, js, tmp);
      }
      ++js;
      ks = save_step(js);
    }
    bool fin = true;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      ur[c] = un[c];
      fin &= isfinite(un[c]);
    }
    if (!fin) {
      ret = GBDE_RET_UNSTABLE;
      ++n;
      break;
    }
  }
  if (ret == GBDE_RET_SUCCESS && n < nl + 1) ret = GBDE_RET_MAXITERS;
  // (a timed-out trajectory keeps GBDE_RET_TIMEOUT; its unreached saves are NaN)
  const double t = n == 0 ? t0 : t_end(n - 1);
  finish_sde<N, float>(a, i, ret, js, (int)n, 0, (int)(2 * n), t, GBDE_ALG_EM, h);
}

template <class M, class T>
__device__ void em_all(const KArgs& a) {
  constexpr int N = M::N;
  WorkSource src;
  src.init();
  const uint64_t t_start = a.timeout_ns ? global_ns() : 0;
  int64_t i;
  while ((i = src.next(a)) >= 0) {
    T p[M::NP], u[N];
#pragma unroll
    for (int k = 0; k < M::NP; ++k) p[k] = (T)__ldg(a.p + (size_t)i * M::NP + k);
#pragma unroll
    for (int c = 0; c < N; ++c) u[c] = (T)__ldg(a.u0 + (size_t)i * N + c);
    const double t0 = __ldg(a.t0 + i), tf = __ldg(a.tf + i);
    const double h = a.dt0;
    int js = 0;
    while (js < a.n_save && save_time(a, i, js) <= t0) {
      store_state<N>(a, i, js, u);
      ++js;
    }
    bool bad = !(tf >= t0) || !isfinite(t0) || !isfinite(tf);
#pragma unroll
    for (int c = 0; c < N; ++c) bad |= !isfinite((double)u[c]);
    if (bad) {
      finish_sde<N, T>(a, i, GBDE_RET_INITIALFAILURE, js, 0, 0, 0, t0, GBDE_ALG_EM,
                       __longlong_as_double(0x7ff8000000000000ll));
      continue;
    }
    NormalStream<T> ns;
    ns.init(a.seed, (uint64_t)i);
    if constexpr (sizeof(T) == 4) {
      em_steps_f32<M>(a, i, t0, tf, h, u, p, js, ns, t_start);
      continue;
    }
    int ret = GBDE_RET_SUCCESS;
    int64_t n = 0;
    double t = t0;
    while (t < tf) {
      if (n >= a.maxiters) {
        ret = GBDE_RET_MAXITERS;
        break;
      }
      if (a.timeout_ns && (n & 1023) == 0 && n > 0 && global_ns() - t_start > a.timeout_ns) {
        ret = GBDE_RET_TIMEOUT;
        atomicOr(a.flag, 1);
        break;
      }
      double tn1 = t0 + (double)(n + 1) * h;
      if (tn1 * (1.0 + 1e-14) >= tf || tn1 > tf) tn1 = tf;
      const double hs = tn1 - t;
      const T sq = (T)sqrt(hs), hT = (T)hs;
      T fu[N], gu[N], un[N];
      M::f(fu, u, p);
      M::g(gu, u, p);
#pragma unroll
      for (int c = 0; c < N; ++c) un[c] = u[c] + fu[c] * hT + gu[c] * (sq * ns.next());
      while (js < a.n_save) {
        const double ts = save_time(a, i, js);
        if (!(ts <= tn1)) break;
        if (ts >= tn1) {
          store_state<N>(a, i, js, un);
        } else {
          const T th = (T)((ts - t) / hs);
          T tmp[N];
#pragma unroll
          for (int c = 0; c < N; ++c) tmp[c] = u[c] + th * (un[c] - u[c]);
          store_state<N>(a, i, js, tmp);
        }
        ++js;
      }
      bool fin = true;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        u[c] = un[c];
        fin &= isfinite((double)un[c]);
      }
      t = tn1;
      ++n;
      if (!fin) {
        ret = GBDE_RET_UNSTABLE;
        break;
      }
    }
    finish_sde<N, T>(a, i, ret, js, (int)n, 0, (int)(2 * n), t, GBDE_ALG_EM, h);
  }
}

// ------------------------------------------------------------ SRI (RSwM)
constexpr int RSWM_DEPTH = 8;

template <int N, class T>
struct NoiseStack {
  double dt[RSWM_DEPTH];
  T W[RSWM_DEPTH][N], Z[RSWM_DEPTH][N];
  int sp;

  GBDE_D void push(double h, const T* w, const T* z) {
    if (sp == RSWM_DEPTH) {
      // merge the two farthest pieces (adjacent in time) to make room
      dt[0] += dt[1];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        W[0][c] += W[1][c];
        Z[0][c] += Z[1][c];
      }
      for (int k = 1; k < RSWM_DEPTH - 1; ++k) {
        dt[k] = dt[k + 1];
#pragma unroll
        for (int c = 0; c < N; ++c) {
          W[k][c] = W[k + 1][c];
          Z[k][c] = Z[k + 1][c];
        }
      }
      sp = RSWM_DEPTH - 1;
    }
    dt[sp] = h;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      W[sp][c] = w[c];
      Z[sp][c] = z[c];
    }
    ++sp;
  }

  // Increments over the next hs time units (consumes / splits pieces,
  // draws fresh normals past the stored future).
  GBDE_D void take(double hs, T* w, T* z, NormalStream<T>& ns) {
#pragma unroll
    for (int c = 0; c < N; ++c) w[c] = z[c] = T(0);
    double acc = 0.0;
    while (true) {
      const double r = hs - acc;
      if (!(r > 1e-14 * hs)) break;
      if (sp > 0) {
        const int k = sp - 1;
        if (dt[k] <= r * (1.0 + 1e-12)) {
          acc += dt[k];
#pragma unroll
          for (int c = 0; c < N; ++c) {
            w[c] += W[k][c];
            z[c] += Z[k][c];
          }
          --sp;
        } else {
          const double frac = r / dt[k];
          const T sd = (T)sqrt(r * (dt[k] - r) / dt[k]);
#pragma unroll
          for (int c = 0; c < N; ++c) {
            const T wr = W[k][c] * (T)frac + sd * ns.next();
            const T zr = Z[k][c] * (T)frac + sd * ns.next();
            w[c] += wr;
            z[c] += zr;
            W[k][c] -= wr;
            Z[k][c] -= zr;
          }
          dt[k] -= r;
          acc = hs;
        }
      } else {
        // FP32 state: the square root on the FP32 pipe (GB300's FP64 pipe is
        // 1/61 of its rate); FP64 state keeps the FP64 square root
        T sq;
        if constexpr (sizeof(T) == 4) sq = __fsqrt_rn((float)r);
        else sq = (T)sqrt(r);
#pragma unroll
        for (int c = 0; c < N; ++c) {
          w[c] += sq * ns.next();
          z[c] += sq * ns.next();
        }
        acc = hs;
      }
    }
  }
};

// Which stages of a 4-stage SRI table (tableaus.h SosriTab / Sriw1Tab) need
// an evaluation: f at H0_i when alpha_i or a later A0 / A1 column uses it, g at
// H1_i when a beta or a later B0 / B1 column does; a stage whose H0 (H1) row
// is empty sits at X and reuses stage 1's f (g).
template <class Tab>
struct SriUse {
  static constexpr bool row_zero(const double (&r)[4]) {
    return r[0] == 0.0 && r[1] == 0.0 && r[2] == 0.0 && r[3] == 0.0;
  }
  static constexpr bool h0_at_x(int i) {
    return i == 0 || (row_zero(Tab::A0[i]) && row_zero(Tab::B0[i]));
  }
  static constexpr bool h1_at_x(int i) {
    return i == 0 || (row_zero(Tab::A1[i]) && row_zero(Tab::B1[i]));
  }
  static constexpr bool f_used(int i) {
    bool u = Tab::al[i] != 0.0;
    for (int k = i + 1; k < 4; ++k) u = u || Tab::A0[k][i] != 0.0 || Tab::A1[k][i] != 0.0;
    return u;
  }
  static constexpr bool g_used(int i) {
    bool u = false;
    for (int q = 0; q < 4; ++q) u = u || Tab::b[q][i] != 0.0;
    for (int k = i + 1; k < 4; ++k) u = u || Tab::B0[k][i] != 0.0 || Tab::B1[k][i] != 0.0;
    return u;
  }
  // f evaluations per step
  static constexpr int n_f() {
    int n = 1;
    for (int i = 1; i < 4; ++i) n += (f_used(i) && !h0_at_x(i)) ? 1 : 0;
    return n;
  }
};

// Compile-time loop: f(IntC<I>) for I = B .. E-1, so that table entries are
// read as constants (and zero entries drop out).  (No <type_traits>: the
// runtime-compiled kernels include this header under NVRTC.)
template <int I>
struct IntC {
  static constexpr int value = I;
};
template <int B, int E, class F>
GBDE_D void static_for(F&& f) {
  if constexpr (B < E) {
    f(IntC<B>{});
    static_for<B + 1, E>(f);
  }
}

// Stage argument X + h sum_j A[i][j] F[j] + s sum_j B[i][j] G[j] (s: I10/h per
// component for H0, sqrt(h) for H1); only the nonzero entries are summed.
template <class Tab, int I, bool H0, int N, class T>
GBDE_D void sri_arg(T* Y, const T* u, const T (*F)[N], const T (*G)[N], T hT, const T* s0,
                    T s1) {
#pragma unroll
  for (int c = 0; c < N; ++c) {
    T af = T(0), bg = T(0);
    static_for<0, I>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      constexpr double a = H0 ? Tab::A0[I][j] : Tab::A1[I][j];
      constexpr double b = H0 ? Tab::B0[I][j] : Tab::B1[I][j];
      if constexpr (a != 0.0) af += T(a) * F[j][c];
      if constexpr (b != 0.0) bg += T(b) * G[j][c];
    });
    Y[c] = u[c] + af * hT + bg * (H0 ? s0[c] : s1);
  }
}

// The drift and diffusion stage values F[i] = f(H0_i), G[i] = g(H1_i) of one
// SRI step (I10h = I10 / h per component).
template <class Tab, class M, class T>
GBDE_D void sri_stages(T (*F)[M::N], T (*G)[M::N], const T* u, const T* p, T hT, T sqh,
                       const T* I10h) {
  constexpr int N = M::N;
  using U = SriUse<Tab>;
  M::f(F[0], u, p);
  M::g(G[0], u, p);
  static_for<1, 4>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    if constexpr (U::f_used(i)) {
      if constexpr (U::h0_at_x(i)) {
#pragma unroll
        for (int c = 0; c < N; ++c) F[i][c] = F[0][c];
      } else {
        T Y[N];
        sri_arg<Tab, i, true, N, T>(Y, u, F, G, hT, I10h, sqh);
        M::f(F[i], Y, p);
      }
    }
    if constexpr (U::g_used(i)) {
      if constexpr (U::h1_at_x(i)) {
#pragma unroll
        for (int c = 0; c < N; ++c) G[i][c] = G[0][c];
      } else {
        T Y[N];
        sri_arg<Tab, i, false, N, T>(Y, u, F, G, hT, I10h, sqh);
        M::g(G[i], Y, p);
      }
    }
  });
}

template <class M, class T, bool MIXED, class Tab, int ALG>
__device__ void sri_all(const KArgs& a) {
  constexpr int N = M::N;
  WorkSource src;
  src.init();
  const uint64_t t_start = a.timeout_ns ? global_ns() : 0;
  int64_t i;
  NoiseStack<N, T> stk;
  while ((i = src.next(a)) >= 0) {
    T p[M::NP], u[N];
#pragma unroll
    for (int k = 0; k < M::NP; ++k) p[k] = (T)__ldg(a.p + (size_t)i * M::NP + k);
#pragma unroll
    for (int c = 0; c < N; ++c) u[c] = (T)__ldg(a.u0 + (size_t)i * N + c);
    const double t0 = __ldg(a.t0 + i), tf = __ldg(a.tf + i);
    int js = 0;
    while (js < a.n_save && save_time(a, i, js) <= t0) {
      store_state<N>(a, i, js, u);
      ++js;
    }
    bool bad = !(tf >= t0) || !isfinite(t0) || !isfinite(tf);
#pragma unroll
    for (int c = 0; c < N; ++c) bad |= !isfinite((double)u[c]);
    if (bad) {
      finish_sde<N, T>(a, i, GBDE_RET_INITIALFAILURE, js, 0, 0, 0, t0, ALG,
                       __longlong_as_double(0x7ff8000000000000ll));
      continue;
    }
    NormalStream<T> ns;
    ns.init(a.seed, (uint64_t)i);
    stk.sp = 0;
    int nfev = 0, nacc = 0, nrej = 0;
    double t = t0;
    double h, dt1 = __longlong_as_double(0x7ff8000000000000ll);
    if (a.pred_dt != nullptr && a.pred_dt[i] > 0.f) {
      h = fmin((double)a.pred_dt[i], tf - t0);
    } else if (a.dt0 > 0.0) {
      h = a.dt0;
    } else {
      T f0[N];
      M::f(f0, u, p);
      ++nfev;
      h = initial_dt<M, T>(u, f0, p, tf - t0, 1, a.abstol, a.reltol, nfev);
    }
    if (a.dtmax > 0.0) h = fmin(h, a.dtmax);
    int ret = GBDE_RET_DEFAULT;
    int64_t iters = 0;
    float lqold = a.ctl.lqoldinit;
    const float atf = (float)a.abstol, rtf = (float)a.reltol;
    if (!(t < tf)) ret = GBDE_RET_SUCCESS;
    while (ret == GBDE_RET_DEFAULT) {
      const double rem = tf - t;
      double hs = h;
      bool last = false;
      if (ord_bits(hs * (1.0 + 1e-10)) >= ord_bits(rem)) {
        hs = rem;
        last = true;
      }
      T dW[N], dZ[N];
      stk.take(hs, dW, dZ, ns);
      // ---- SRI step (with FP32 state the step's powers are FP32 operations)
      T hT, sqh, ih, isqh;
      if constexpr (sizeof(T) == 4) {
        hT = (float)hs;
        sqh = __fsqrt_rn(hT);
        ih = __frcp_rn(hT);
        isqh = __frcp_rn(sqh);
      } else {
        hT = (T)hs;
        sqh = (T)sqrt(hs);
        ih = (T)(1.0 / hs);
        isqh = (T)(1.0 / sqrt(hs));
      }
      T I10[N], I11[N], I111[N], I10h[N];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        I10[c] = T(0.5) * hT * (dW[c] + dZ[c] * T(0.57735026918962576451));
        I11[c] = T(0.5) * (dW[c] * dW[c] - hT);
        I111[c] = (dW[c] * dW[c] * dW[c] - T(3) * hT * dW[c]) * T(1.0 / 6.0);
        I10h[c] = I10[c] * ih;
      }
      T F[4][N], G[4][N], un[N], err[N];
      sri_stages<Tab, M, T>(F, G, u, p, hT, sqh, I10h);
      nfev += SriUse<Tab>::n_f();
#pragma unroll
      for (int c = 0; c < N; ++c) {
        T drift = T(0), ed = T(0), sto = T(0), g3 = T(0), g4 = T(0);
        static_for<0, 4>([&](auto kc) {
          constexpr int k = decltype(kc)::value;
          constexpr double al = Tab::al[k], ale = al - (k == 0 ? 1.0 : 0.0);
          constexpr double b1 = Tab::b[0][k], b2 = Tab::b[1][k], b3 = Tab::b[2][k],
                           b4 = Tab::b[3][k];
          if constexpr (al != 0.0) drift += T(al) * F[k][c];
          // the embedded Euler drift (alpha = e_1) for the error estimate
          if constexpr (ale != 0.0) ed += T(ale) * F[k][c];
          if constexpr (b1 != 0.0 || b2 != 0.0 || b3 != 0.0 || b4 != 0.0) {
            const T w = T(b1) * dW[c] + T(b2) * I11[c] * isqh + T(b3) * I10h[c] +
                        T(b4) * I111[c] * ih;
            sto += w * G[k][c];
          }
          if constexpr (b3 != 0.0) g3 += T(b3) * G[k][c];
          if constexpr (b4 != 0.0) g4 += T(b4) * G[k][c];
        });
        un[c] = u[c] + hT * drift + sto;
        ed *= hT;
        const T en = g3 * I10h[c] + g4 * I111[c] * ih;
        err[c] = (ed < T(0) ? -ed : ed) + (en < T(0) ? -en : en);
      }
      double ms;  // EEst^2
      if constexpr (sizeof(T) == 4) ms = err_ms_f32<N>(err, u, un, atf, rtf);
      else ms = err_ms<N>(err, u, un, a.abstol, a.reltol);
      ++iters;
      // ms <= 1 (ms >= 0; NaN rejects) and the other bookkeeping compares on
      // the integer pipe, as integrate_all
      if (!a.adaptive || mag_bits(ms) <= 0x3FF0000000000000ull) {
        // t + h in FP64 in every precision, as the FP64 oracle forms it
        const double tnew = last ? tf : t + hs;
        const uint64_t tnew_o = ord_bits(tnew);
        while (js < a.n_save) {
          const double ts = save_time(a, i, js);
          const uint64_t ts_o = ord_bits(ts);
          if (ts_o > tnew_o) break;
          if (ts_o == tnew_o) {
            store_state<N>(a, i, js, un);
          } else {
            const T th = (T)((ts - t) / hs);
            T tmp[N];
#pragma unroll
            for (int c = 0; c < N; ++c) tmp[c] = u[c] + th * (un[c] - u[c]);
            store_state<N>(a, i, js, tmp);
          }
          ++js;
        }
        bool fin = true;
#pragma unroll
        for (int c = 0; c < N; ++c) {
          u[c] = un[c];
          fin &= val_finite(un[c]);
        }
        t = tnew;
        if (nacc == 0) dt1 = hs;
        ++nacc;
        if (!fin) ret = GBDE_RET_UNSTABLE;
        else if (last) ret = GBDE_RET_SUCCESS;
        if (a.adaptive) h = hs * f2d_bits(ctl_accept(a.ctl, ms, lqold));
      } else {
        ++nrej;
        stk.push(hs, dW, dZ);
        h = hs * f2d_bits(ctl_reject(a.ctl, ms));
      }
      if (a.dtmax > 0.0 && ord_bits(h) > ord_bits(a.dtmax)) h = a.dtmax;
      if (ret == GBDE_RET_DEFAULT) {
        if (iters >= a.maxiters) ret = GBDE_RET_MAXITERS;
        else if (a.adaptive && dt_too_small(h, a.dtmin, t))
          ret = GBDE_RET_DTLESSTHANMIN;
        else if (a.timeout_ns && (iters & 31) == 0 && global_ns() - t_start > a.timeout_ns) {
          ret = GBDE_RET_TIMEOUT;
          atomicOr(a.flag, 1);
        }
      }
    }
    finish_sde<N, T>(a, i, ret, js, nacc, nrej, nfev, t, ALG, dt1);
  }
}

}  // namespace gbde
