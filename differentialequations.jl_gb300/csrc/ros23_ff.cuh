// ros23_ff.cuh -- Rosenbrock23 in FP32 pairs (the F32X2 precision) for models
// of up to three states.
//
// Same method as Ros23Alg (rosenbrock.cuh; OrdinaryDiffEq's Rosenbrock23,
// test/qa/qa.jl:98): Shampine and Reichelt's 2(3) W-method with W = I - h d J,
// three solves, the error estimate h/6 (k1 - 2 k2 + k3) and the 2nd-order dense
// output.  The work is placed as in RodasFF (rodas_ff.cuh): the Jacobian, W and
// its partial-pivot LU are FP64, built afresh on every attempt from the FP64
// value of the state; the factors reach the pair solves through the
// integer-pipe split (FfLU); state, stages, right-hand sides and the stage
// combinations are pairs; the norm's ratios are FP32 on the leading parts with
// their squares accumulated in FP64.
#pragma once
#include "rodas_ff.cuh"

namespace gbde {

template <class M>
struct Ros23FF {
  using T = ff;
  static constexpr int ORDER = 2, ALG_ID = GBDE_ALG_ROSENBROCK23, N = M::N;
  ff uu[N], un[N], F0[N], F2[N], k1[N], k2[N];
  double pd[M::NP];

  GBDE_D const ff* u() const { return uu; }
  GBDE_D const ff* unew() const { return un; }
  GBDE_D const ff* f0() const { return F0; }

  GBDE_D void init(const ff* u0, const ff* p, int& nf) {
#pragma unroll
    for (int k = 0; k < M::NP; ++k) pd[k] = (double)p[k];
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = u0[c];
    M::f(F0, uu, p);
    ++nf;
  }

  GBDE_D double attempt(double dt, const ff* p, double abstol, double reltol, int& nf) {
    using namespace tab::ros23;
    SmallLU<N> W;
    {
      double ud[N], J[N][N];
#pragma unroll
      for (int c = 0; c < N; ++c) ud[c] = f2d_bits(uu[c].hi) + f2d_bits(uu[c].lo);
      M::jac(J, ud, pd);
      const double hd = dt * d;
#pragma unroll
      for (int r = 0; r < N; ++r)
#pragma unroll
        for (int c = 0; c < N; ++c) W.A[r][c] = (r == c ? 1.0 : 0.0) - hd * J[r][c];
    }
    W.factor();
    FfLU<N> L;
    L.from(W);
    constexpr ff E32 = ff(e32), NE32 = ff(-e32), SIXTH = ff(1.0 / 6.0);
    const ff two(2.0f, 0.0f), ntwo(-2.0f, 0.0f);
    const ff h = ff_split(dt), hh(0.5f * h.hi, 0.5f * h.lo);  // h / 2, exactly
    // k1 = W^-1 f(u0)
#pragma unroll
    for (int c = 0; c < N; ++c) k1[c] = F0[c];
    L.solve(k1);
    // k2 = W^-1 (f(u0 + h/2 k1) - k1) + k1
    ff y[N], F1[N];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      FfAcc a;
      a.set(uu[c]);
      a.fma(hh, k1[c]);
      y[c] = a.get();
    }
    M::f(F1, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) k2[c] = F1[c] - k1[c];
    L.solve(k2);
    // u1 = u0 + h k2
#pragma unroll
    for (int c = 0; c < N; ++c) {
      k2[c] = k2[c] + k1[c];
      FfAcc a;
      a.set(uu[c]);
      a.fma(h, k2[c]);
      un[c] = a.get();
    }
    M::f(F2, un, p);
    nf += 2;
    // k3 = W^-1 (f(u1) - e32 (k2 - F1) - 2 (k1 - F0))
    ff k3[N];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      FfAcc a;
      a.set(F2[c]);
      a.fma(NE32, k2[c]);
      a.fma(E32, F1[c]);
      a.fma(ntwo, k1[c]);
      a.fma(two, F0[c]);
      k3[c] = a.get();
    }
    L.solve(k3);
    // error estimate h/6 (k1 - 2 k2 + k3); norm ratios in FP32, squares in FP64
    const ff h6 = h * SIXTH;
    const float atf = tol_f32(abstol), rtf = tol_f32(reltol);
    double ms = 0.0;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      FfAcc a;
      a.set(k1[c]);
      a.fma(ntwo, k2[c]);
      a.add(k3[c]);
      const ff err = a.get() * h6;
      const float m = fmaxf(fabsf(uu[c].hi), fabsf(un[c].hi));
      const double e = f2d_bits(norm_ratio(err.hi, fmaf(rtf, m, atf)));
      ms = fma(e, e, ms);
    }
    return ms * (1.0 / N);
  }

  // y(theta) = u0 + h (w1 k1 + w2 k2), w1 = theta (1 - theta) / (1 - 2d),
  // w2 = theta (theta - 2d) / (1 - 2d) (as Ros23Alg::interp), in pairs
  GBDE_D void interp(double th, double dt, ff* out, const ff*, int&) {
    using namespace tab::ros23;
    constexpr ff DEN = ff(1.0 / (1.0 - 2.0 * d)), D2 = ff(2.0 * d);
    const ff t = ff_split(th), h = ff_split(dt);
    const ff w1 = h * (t * (ff(1.0f, 0.0f) - t) * DEN), w2 = h * (t * (t - D2) * DEN);
#pragma unroll
    for (int c = 0; c < N; ++c) {
      FfAcc a;
      a.set(uu[c]);
      a.fma(w1, k1[c]);
      a.fma(w2, k2[c]);
      out[c] = a.get();
    }
  }

  GBDE_D void accept(const ff*, int&) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = un[c];
      F0[c] = F2[c];
    }
  }
};

// The Rosenbrock23 stepper for precision T: the pair stepper above for F32X2
// models of up to three states, Ros23Alg otherwise.
template <class M, class T, bool PAIR = is_ff<T>::value && (M::N <= 3)>
struct Ros23Sel {
  using type = Ros23Alg<M, T>;
};
template <class M, class T>
struct Ros23Sel<M, T, true> {
  using type = Ros23FF<M>;
};
template <class M, class T>
using Ros23A = typename Ros23Sel<M, T>::type;

}  // namespace gbde
