// autoswitch.cuh -- AutoTsit5(stiff method): per-trajectory run-time switching
// between Tsit5 and a Rosenbrock method (the reference's AutoTsit5(
// Rosenbrock23()), test/qa/qa.jl:15; OrdinaryDiffEq's composite algorithms,
// not vendored in the reference).
//
// Every attempted step leaves a stiffness estimate: Tsit5's from its last two
// stages (Hairer & Wanner II, IV.2, infinity norm: Tsit5Alg<..., EIG>), the
// Rosenbrock method's the infinity norm of the Jacobian it used.  Before every
// attempt after the first, the switching rule with AutoSwitch's published
// defaults (maxstiffstep = 10, maxnonstiffstep = 3, nonstifftol = stifftol =
// 9/10, dtfac = 2, stiffalgfirst = false) decides the method:
//   stiffness = |eig * dt / 3.5068|          (3.5068: Tsit5's stability size
//                                             on the negative real axis)
//   stiff     = stiffness > 9/10
//   count     = stiff ? (count < 0 ? 1 : count + 1) : (count > 0 ? -1 : count - 1)
//   Tsit5 and count > 10   -> the stiff method, dt * 2
//   stiff method and count < -3 -> Tsit5, dt / 2
// A switch continues at the current accepted state with its f(u) (evaluated
// anew only when the stiff method does not hold it: Rodas re-evaluates f at
// the start of each attempt); the PI controller keeps its memory and takes the
// new method's exponents (KArgs::ctl_stiff for the stiff method).  Saves use the dense
// output of the method that took the step.  AutoSwitch's successive_switches
// limit on skipping the error test is not restated: every step is error
// controlled.
#pragma once
#include "explicit_rk.cuh"
#include "rosenbrock.cuh"

namespace gbde {

constexpr double kTsit5StabilitySize = 3.5068;

template <class M, class T, class S>
struct AutoSwitchAlg {
  static constexpr int ORDER = 5, N = M::N;  // Tsit5 first: its order for the starting step
  static constexpr int ALG_ID = GBDE_ALG_TSIT5;
  Tsit5Alg<M, T, true> ns;
  S st;
  bool stiff;  // the method of the current step
  int count;   // successive stiff (> 0) or non-stiff (< 0) estimates
  double eig;  // the last attempt's estimate

  GBDE_D const T* u() const { return stiff ? st.u() : ns.u(); }
  GBDE_D const T* unew() const { return stiff ? st.unew() : ns.unew(); }
  GBDE_D const T* f0() const { return stiff ? st.f0() : ns.f0(); }
  GBDE_D int method() const { return stiff ? S::ALG_ID : GBDE_ALG_TSIT5; }

  GBDE_D void init(const T* u0, const T* p, int& nf) {
    ns.init(u0, p, nf);
    stiff = false;
    count = 0;
    eig = 0.0;
  }

  GBDE_D double attempt(double dt, const T* p, double abstol, double reltol, int& nf) {
    double ms;
    if (stiff) {
      ms = st.attempt(dt, p, abstol, reltol, nf);
      eig = st.jac_norm();
    } else {
      ms = ns.attempt(dt, p, abstol, reltol, nf);
      eig = ns.eig;
    }
    return ms;
  }

  GBDE_D void interp(double th, double dt, T* out, const T* p, int& nf) {
    if (stiff) st.interp(th, dt, out, p, nf);
    else ns.interp(th, dt, out, p, nf);
  }

  GBDE_D void accept(const T* p, int& nf) {
    if (stiff) st.accept(p, nf);
    else ns.accept(p, nf);
  }

  // The switching rule, before an attempt of step size dt; returns the step
  // size to attempt.
  GBDE_D double choose(double dt, const T* p, int& nf) {
    const double stiffness = fabs(eig * dt / kTsit5StabilitySize);
    const bool s = stiffness > 0.9;  // NaN: not stiff
    count = s ? (count < 0 ? 1 : count + 1) : (count > 0 ? -1 : count - 1);
    if (!stiff && count > 10) {
      T uc[N], fc[N];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        uc[c] = ns.u()[c];
        fc[c] = ns.f0()[c];
      }
      st.init_from(uc, fc, p);
      stiff = true;
      return dt * 2.0;
    }
    if (stiff && count < -3) {
      T uc[N], fc[N];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        uc[c] = st.u()[c];
        fc[c] = st.f0()[c];
      }
      if (st.f0_valid()) ns.init_from(uc, fc, p);
      else ns.init(uc, p, nf);
      stiff = false;
      return dt / 2.0;
    }
    return dt;
  }
};

template <class M, class T, class S>
struct switching<AutoSwitchAlg<M, T, S>> {
  static constexpr bool v = true;
};

}  // namespace gbde
