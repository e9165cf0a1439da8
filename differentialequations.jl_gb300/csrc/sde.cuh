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
                             const float* p, int js, NormalStream<float>& ns) {
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
  const double t = n == 0 ? t0 : t_end(n - 1);
  finish_sde<N, float>(a, i, ret, js, (int)n, 0, (int)(2 * n), t, GBDE_ALG_EM, h);
}

template <class M, class T>
__device__ void em_all(const KArgs& a) {
  constexpr int N = M::N;
  WorkSource src;
  src.init();
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
      em_steps_f32<M>(a, i, t0, tf, h, u, p, js, ns);
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

template <class M, class T, bool MIXED>
__device__ void sri_all(const KArgs& a) {
  using namespace tab::sriw1;
  constexpr int N = M::N;
  WorkSource src;
  src.init();
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
      finish_sde<N, T>(a, i, GBDE_RET_INITIALFAILURE, js, 0, 0, 0, t0, GBDE_ALG_SOSRI,
                       __longlong_as_double(0x7ff8000000000000ll));
      continue;
    }
    NormalStream<T> ns;
    ns.init(a.seed, (uint64_t)i);
    stk.sp = 0;
    int nfev = 0, nacc = 0, nrej = 0;
    double t = t0, tlo = 0.0;
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
      // ---- SRIW1 step (with FP32 state the step's powers are FP32 operations)
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
      T F1[N], F2[N], G1[N], G2[N], G3[N], G4[N], Y[N], un[N], err[N];
      M::f(F1, u, p);
      M::g(G1, u, p);
      T I10[N], I11[N], I111[N];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        I10[c] = T(0.5) * hT * (dW[c] + dZ[c] * T(0.57735026918962576451));
        I11[c] = T(0.5) * (dW[c] * dW[c] - hT);
        I111[c] = (dW[c] * dW[c] * dW[c] - T(3) * hT * dW[c]) * T(1.0 / 6.0);
      }
#pragma unroll
      for (int c = 0; c < N; ++c) Y[c] = u[c] + T(A0_21) * F1[c] * hT + T(B0_21) * G1[c] * I10[c] * ih;
      M::f(F2, Y, p);
#pragma unroll
      for (int c = 0; c < N; ++c) Y[c] = u[c] + T(A1_21) * F1[c] * hT + T(B1_21) * G1[c] * sqh;
      M::g(G2, Y, p);
#pragma unroll
      for (int c = 0; c < N; ++c) Y[c] = u[c] + T(A1_31) * F1[c] * hT + T(B1_31) * G1[c] * sqh;
      M::g(G3, Y, p);
#pragma unroll
      for (int c = 0; c < N; ++c)
        Y[c] = u[c] + T(A1_43) * F1[c] * hT +
               (T(B1_41) * G1[c] + T(B1_42) * G2[c] + T(B1_43) * G3[c]) * sqh;
      M::g(G4, Y, p);
      nfev += 2;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const T w1 = T(b1_1) * dW[c] + T(b2_1) * I11[c] * isqh + T(b3_1) * I10[c] * ih + T(b4_1) * I111[c] * ih;
        const T w2 = T(b1_2) * dW[c] + T(b2_2) * I11[c] * isqh + T(b3_2) * I10[c] * ih + T(b4_2) * I111[c] * ih;
        const T w3 = T(b1_3) * dW[c] + T(b2_3) * I11[c] * isqh + T(b3_3) * I10[c] * ih + T(b4_3) * I111[c] * ih;
        const T w4 = T(b1_4) * dW[c] + T(b2_4) * I11[c] * isqh + T(b3_4) * I10[c] * ih + T(b4_4) * I111[c] * ih;
        un[c] = u[c] + hT * (T(al1) * F1[c] + T(al2) * F2[c]) + w1 * G1[c] + w2 * G2[c] +
                w3 * G3[c] + w4 * G4[c];
        const T ed = hT * (T(al1 - 1.0) * F1[c] + T(al2) * F2[c]);
        const T en = (T(b3_1) * G1[c] + T(b3_2) * G2[c] + T(b3_3) * G3[c] + T(b3_4) * G4[c]) * I10[c] * ih +
                     (T(b4_1) * G1[c] + T(b4_2) * G2[c] + T(b4_3) * G3[c] + T(b4_4) * G4[c]) * I111[c] * ih;
        err[c] = (ed < T(0) ? -ed : ed) + (en < T(0) ? -en : en);
      }
      double ms;  // EEst^2
      if constexpr (sizeof(T) == 4) ms = err_ms_f32<N>(err, u, un, atf, rtf);
      else ms = err_ms<N>(err, u, un, a.abstol, a.reltol);
      ++iters;
      // ms <= 1 (ms >= 0; NaN rejects) and the other bookkeeping compares on
      // the integer pipe, as integrate_all
      if (!a.adaptive || mag_bits(ms) <= 0x3FF0000000000000ull) {
        double tnew;
        if (last) {
          tnew = tf;
          tlo = 0.0;
        } else if (MIXED) {
          // Fast2Sum on the operands ordered by magnitude
          const bool tb = mag_bits(t) >= mag_bits(hs);
          const double big = tb ? t : hs, small = tb ? hs : t;
          const double s = big + small;
          double e = small - (s - big);
          e += tlo;
          tnew = s + e;
          tlo = e - (tnew - s);
        } else {
          tnew = t + hs;
        }
        const uint64_t tnew_o = ord_bits(tnew);
        while (js < a.n_save) {
          const double ts = save_time(a, i, js);
          const uint64_t ts_o = ord_bits(ts);
          if (ts_o > tnew_o) break;
          if (ts_o == tnew_o) {
            store_state<N>(a, i, js, un);
          } else {
            const T th = (T)(((ts - t) - tlo) / hs);
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
      }
    }
    finish_sde<N, T>(a, i, ret, js, nacc, nrej, nfev, t + tlo, GBDE_ALG_SOSRI, dt1);
  }
}

}  // namespace gbde
