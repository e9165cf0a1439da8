// solver.cuh -- the per-trajectory integration driver shared by every
// ODE method: step-size controller, error norm, initial dt, saveat writer,
// tf handling, return codes and the work source (plain launch or persistent
// device queue).
//
// The driver replaces, per trajectory, OrdinaryDiffEq's solve! loop
// (perform_step!, the PI controller, savevalues!) that SciMLBase's
// EnsembleThreads maps over trajectories (EnsembleThreads, test/qa/qa.jl:56;
// the controller accessors it exposes are get_proposed_dt / set_proposed_dt!
// / auto_dt_reset!, qa.jl:151,187,135).  Controller formulas follow
// Hairer-Norsett-Wanner I, Sec. II.4 and Gustafsson's PI control:
//     q11 = EEst^beta1,  q = q11 / qold^beta2,
//     q   = clamp(q / gamma, 1/qmax, 1/qmin)
//     accept (EEst <= 1): q = 1 if qsteady_min <= q <= qsteady_max;
//                         dt <- dt / q;  qold = max(EEst, qoldinit)
//     reject:             dt <- dt / min(1/qmin, q11 / gamma)
// with the scaled RMS norm
//     EEst = sqrt(mean_i (err_i / (abstol + reltol max(|u_i|, |unew_i|)))^2).
#pragma once
#include "common.cuh"
#include "controller.h"
#include "models.cuh"

namespace gbde {

// Kernel arguments (passed by value; lives in the constant bank).
struct KArgs {
  int64_t N;
  int32_t n_save, save_kind;
  const double* p;
  const double* u0;
  const double* t0;
  const double* tf;
  const double* saveat;
  void* u_out;
  int32_t out_f32;
  int32_t* retcode;
  int32_t* naccept;
  int32_t* nreject;
  int32_t* nf;
  double* t_end;
  int32_t* method_out;
  double reltol, abstol, dt0, dtmin, dtmax;
  int64_t maxiters;
  int32_t adaptive;
  double qmin, qmax, gamma, beta1, beta2, qsteady_min, qsteady_max, qoldinit;
  uint64_t seed;
  unsigned long long* queue;  // persistent work counter (NULL = plain launch)
  const int32_t* order;       // optional trajectory order for the queue
  uint64_t timeout_ns;        // 0 = no deadline
  int32_t* flag;              // device status word (bit 0: deadline hit)
  const float* pred_dt;       // optional predicted first dt per trajectory
  CtlK ctl;                   // step-size controller constants (controller.h)
  CtlK ctl_stiff;             // the stiff method's, in a switching composite (autoswitch.cuh)
  double* dt_first;           // optional: size of the first accepted step
  int32_t chunk;              // persistent queue positions per fetch (>= 1)
  const double* dt_init;      // optional: starting step per trajectory (k_init_dt)
  double* red;                // optional: [2][n_save][N] sums and sums of squares of the
                              // saved states over trajectories (u_out may then be NULL)
  double* ev_t;               // optional: [N][ev_cap] times of the saves at callback events
  void* ev_u;                 // optional: [N][ev_cap][n_state] their states (out_f32's type)
  int32_t* ev_n;              // optional: [N] event saves made (callback kernels only)
  int32_t ev_cap;             // event saves per trajectory the buffers hold
};

GBDE_D uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ----------------------------------------------------------- work source
// Plain launch: each thread takes its own index once.  Persistent launch:
// threads that need work take consecutive indices from a global counter
// with one atomic per group of converged lanes (warp-aggregated: the lowest
// active lane adds for all of them and broadcasts the base).
// With chunk c > 1 a thread takes c consecutive queue positions per fetch.
struct WorkSource {
  int64_t first;
  bool used;
  unsigned long long cur, end;  // this thread's remaining chunk [cur, end)
  GBDE_D void init() {
    first = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    used = false;
    cur = end = 0;
  }
  GBDE_D int64_t next(const KArgs& a) {
    if (a.queue == nullptr) {
      if (used) return -1;
      used = true;
      if (first >= a.N) return -1;
      return a.order ? (int64_t)a.order[first] : first;
    }
    if (cur >= end) {
      const unsigned long long c = a.chunk > 1 ? (unsigned long long)a.chunk : 1ull;
      const unsigned m = __activemask();
      const int lane = (int)(threadIdx.x & 31u);
      const int leader = __ffs((int)m) - 1;
      const unsigned rank = (unsigned)__popc(m & ((1u << lane) - 1u));
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(a.queue, (unsigned long long)__popc(m) * c);
      base = __shfl_sync(m, base, leader);
      cur = base + rank * c;
      end = cur + c;
    }
    const unsigned long long idx = cur++;
    if (idx >= (unsigned long long)a.N) {
      cur = end = ~0ull;  // exhausted
      return -1;
    }
    return a.order ? (int64_t)a.order[idx] : (int64_t)idx;
  }
};

// dt < dtmin or dt <= 4 eps |t| (no representable progress), compared as
// integers: 4 eps |t| = |t| 2^-50 is |t|'s bit pattern with the exponent
// lowered by 50 (taken as 0 for |t| < 2^-972).  dt and dtmin are not NaN.
GBDE_D bool dt_too_small(double dt, double dtmin, double t) {
  if (ord_bits(dt) < ord_bits(dtmin)) return true;
  const uint64_t tb = mag_bits(t), sh = 50ull << 52;
  const uint64_t lim = tb > sh ? tb - sh : 0ull;
  return (__double_as_longlong(dt) < 0) || mag_bits(dt) <= lim;
}

// ------------------------------------------------------------- saving
GBDE_D double save_time(const KArgs& a, int64_t i, int j) {
  return a.save_kind == GBDE_SAVE_GRID ? __ldg(a.saveat + j)
                                       : __ldg(a.saveat + (size_t)i * a.n_save + j);
}

// In-kernel reduction of a saved state: FP64 atomics into the sums of save
// point j (the order of the additions is not fixed, so sums agree with a
// sequential sum to FP64 rounding).
GBDE_D void reduce_add(const KArgs& a, int j, int c, int n_state, double x) {
  atomicAdd(&a.red[(size_t)j * n_state + c], x);
  atomicAdd(&a.red[((size_t)a.n_save + j) * n_state + c], x * x);
}

template <int N, class T>
GBDE_D void store_state(const KArgs& a, int64_t i, int j, const T* v) {
  if (a.red) {
#pragma unroll
    for (int c = 0; c < N; ++c) reduce_add(a, j, c, N, (double)v[c]);
  }
  if (a.u_out == nullptr) return;
  const size_t base = ((size_t)i * a.n_save + j) * N;
  if (a.out_f32) {
    float* o = (float*)a.u_out + base;
    if constexpr (N % 4 == 0) {
#pragma unroll
      for (int c = 0; c < N; c += 4)
        *reinterpret_cast<float4*>(o + c) =
            make_float4((float)v[c], (float)v[c + 1], (float)v[c + 2], (float)v[c + 3]);
    } else if constexpr (N % 2 == 0) {
#pragma unroll
      for (int c = 0; c < N; c += 2)
        *reinterpret_cast<float2*>(o + c) = make_float2((float)v[c], (float)v[c + 1]);
    } else {
#pragma unroll
      for (int c = 0; c < N; ++c) o[c] = (float)v[c];
    }
  } else {
    double* o = (double*)a.u_out + base;
    if constexpr (N % 2 == 0) {
#pragma unroll
      for (int c = 0; c < N; c += 2)
        *reinterpret_cast<double2*>(o + c) = make_double2((double)v[c], (double)v[c + 1]);
    } else {
#pragma unroll
      for (int c = 0; c < N; ++c) o[c] = (double)v[c];
    }
  }
}

// --------------------------------------------------------- error norm
// Mean square of the scaled error, ms = EEst^2 (the accept test is ms <= 1).
// Each err_c / sc_c uses the Newton-refined reciprocal of controller.h
// instead of an IEEE division.
// err_ms with FP32 state: the ratios err_c / (abstol + reltol max(|u_c|,
// |u1_c|)) are FP32 operations, their squares accumulate in FP64.
template <int N>
GBDE_D double err_ms_f32(const float* err, const float* u, const float* unew, float atf,
                         float rtf) {
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < N; ++c) {
    const float m = fmaxf(fabsf(u[c]), fabsf(unew[c]));
    const double e = f2d_bits(__fdiv_rn(err[c], fmaf(rtf, m, atf)));
    s = fma(e, e, s);
  }
  return s * (1.0 / N);
}

template <int N, class T>
GBDE_HD double err_ms(const T* err, const T* u, const T* unew, double abstol, double reltol) {
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(T) == 4)  // FP32 state
    return err_ms_f32<N>(err, u, unew, (float)abstol, (float)reltol);
#endif
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < N; ++c) {
    const double sc = abstol + reltol * fmax(fabs((double)u[c]), fabs((double)unew[c]));
    const double e = (double)err[c] * rcp64(sc);
    s += e * e;
  }
  return s * (1.0 / N);
}

template <int N, class T>
GBDE_HD double err_norm(const T* err, const T* u, const T* unew, double abstol, double reltol) {
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < N; ++c) {
    const double sc = abstol + reltol * fmax(fabs((double)u[c]), fabs((double)unew[c]));
    const double e = (double)err[c] / sc;
    s += e * e;
  }
  return sqrt(s / N);
}

// Hairer-Wanner starting step (HNW I, Sec. II.4): mean squares of the
// scaled u0, f0 and of one explicit Euler trial step's change in f, then
// hw_h0 / hw_dt (controller.h).
template <class M, class T>
GBDE_D double initial_dt(const T* u0, const T* f0, const T* p, double tspan, int order,
                         double abstol, double reltol, int& nf) {
  constexpr int N = M::N;
  double s0 = 0.0, s1 = 0.0, rs[N];
#pragma unroll
  for (int c = 0; c < N; ++c) {
    rs[c] = rcp64(abstol + fabs((double)u0[c]) * reltol);
    const double x = (double)u0[c] * rs[c], y = (double)f0[c] * rs[c];
    s0 += x * x;
    s1 += y * y;
  }
  s0 *= 1.0 / N;
  s1 *= 1.0 / N;
  const double h0 = hw_h0(s0, s1, tspan);
  T u1[N], f1[N];
#pragma unroll
  for (int c = 0; c < N; ++c) u1[c] = u0[c] + T(h0) * f0[c];
  M::f(f1, u1, p);
  ++nf;
  double s2 = 0.0;
#pragma unroll
  for (int c = 0; c < N; ++c) {
    const double y = ((double)f1[c] - (double)f0[c]) * rs[c];
    s2 += y * y;
  }
  return hw_dt(h0, s1, s2 * (1.0 / N), tspan, order);
}

// Pre-pass: the Hairer-Wanner starting step of every trajectory, one thread
// each, all lanes converged.  Same loads, Alg::init and initial_dt as the
// step kernel, so the step kernel starts from the identical value.
template <class Alg, class M, class T>
__device__ void init_dt_all(const KArgs& a, double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.N;
       i += (int64_t)gridDim.x * blockDim.x) {
    T p[M::NP], u0[M::N];
#pragma unroll
    for (int k = 0; k < M::NP; ++k) p[k] = (T)__ldg(a.p + (size_t)i * M::NP + k);
#pragma unroll
    for (int c = 0; c < M::N; ++c) u0[c] = (T)__ldg(a.u0 + (size_t)i * M::N + c);
    const double t0 = __ldg(a.t0 + i), tf = __ldg(a.tf + i);
    bool bad = !(tf > t0) || !isfinite(t0) || !isfinite(tf);
#pragma unroll
    for (int c = 0; c < M::N; ++c) bad |= !isfinite((double)u0[c]);
    double dt = 0.0;
    if (!bad) {
      Alg alg;
      int nf = 0;
      alg.init(u0, p, nf);
      dt = initial_dt<M, T>(alg.u(), alg.f0(), p, tf - t0, Alg::ORDER, a.abstol, a.reltol, nf);
    }
    out[i] = dt;
  }
}
template <class Alg, class M, class T>
__global__ void __launch_bounds__(128) k_init_dt(const KArgs a, double* __restrict__ out) {
  init_dt_all<Alg, M, T>(a, out);
}

// ----------------------------------------------------------- callbacks
// Event handling of the reference's ContinuousCallback, DiscreteCallback,
// VectorContinuousCallback and CallbackSet (qa.jl:24,36,124,26; exercised by
// test/core.jl:60-79).  The precompiled kernels use NoCallback and compile none
// of it.  A callback type (runtime-compiled from user source, rtc.cu) provides
//   static constexpr int NC;   continuous conditions: 1 per ContinuousCallback,
//                              len per VectorContinuousCallback, summed over a set
//   static constexpr int ND;   discrete callbacks
//   static void conditions(const double* u, double t, const double* p, double* g);
//   static void affect_c(int idx, double* u, double t, const double* p, bool& terminate);
//   static bool condition_d(int k, const double* u, double t, const double* p);
//   static void affect_d(int k, double* u, double t, const double* p, bool& terminate);
// on FP64 copies of the state and parameters, whatever the precision.
// Continuous: a sign change of condition idx over an accepted step is located
// on the method's dense output by Illinois regula falsi; of several, the
// earliest root is the event.  The integrator moves to the left side of the
// root (the reference's LeftRootFind default), applies affect idx and restarts
// the method there.  Save points up to the event use the step's dense output.
// For the condition that fired, the next step looks for crossings only after
// 1% of its length (the reference's repeat_nudge), so a root is not found
// twice; the other conditions start from their values after the affect.
// Discrete: after an accepted step each condition k that is true applies its
// affect, in order, on the state the previous ones left.
// Event saves (the reference's save_positions; save_c(idx) / save_d(k) give
// the GBDE_SAVE_* bits of continuous condition idx / discrete callback k,
// SAVES their union): (t, u) before an affect, unless a saveat point at
// exactly t was stored at that moment, and (t, u) after it.
struct NoCallback {
  static constexpr int NC = 0, ND = 0, SAVES = 0;
  GBDE_D static int save_c(int) { return 0; }
  GBDE_D static int save_d(int) { return 0; }
  GBDE_D static void conditions(const double*, double, const double*, double*) {}
  GBDE_D static void affect_c(int, double*, double, const double*, bool&) {}
  GBDE_D static bool condition_d(int, const double*, double, const double*) { return false; }
  GBDE_D static void affect_d(int, double*, double, const double*, bool&) {}
};

template <class CB, int N, int NP, class T>
GBDE_D void cb_conditions(const T* u, double t, const T* p, double* g) {
  double ud[N], pd[NP];
#pragma unroll
  for (int c = 0; c < N; ++c) ud[c] = (double)u[c];
#pragma unroll
  for (int k = 0; k < NP; ++k) pd[k] = (double)p[k];
  CB::conditions(ud, t, pd, g);
}

// continuous affect idx on an FP64 copy of u; returns terminate
template <class CB, int N, int NP, class T>
GBDE_D bool cb_affect_c(int idx, T* u, double t, const T* p) {
  double ud[N], pd[NP];
#pragma unroll
  for (int c = 0; c < N; ++c) ud[c] = (double)u[c];
#pragma unroll
  for (int k = 0; k < NP; ++k) pd[k] = (double)p[k];
  bool term = false;
  CB::affect_c(idx, ud, t, pd, term);
#pragma unroll
  for (int c = 0; c < N; ++c) u[c] = (T)ud[c];
  return term;
}

// every discrete callback in order on u; returns (any fired, terminate).
// save(t, ud) makes an event save; `exact`: a saveat point at exactly t was
// stored just before (the first callback to fire then saves nothing before
// its affect).
template <class CB, int N, int NP, class T, class Save>
GBDE_D bool cb_discrete(T* u, double t, const T* p, bool& term, bool exact, Save&& save) {
  double ud[N], pd[NP];
#pragma unroll
  for (int c = 0; c < N; ++c) ud[c] = (double)u[c];
#pragma unroll
  for (int k = 0; k < NP; ++k) pd[k] = (double)p[k];
  bool any = false;
#pragma unroll
  for (int k = 0; k < CB::ND; ++k) {
    if (CB::condition_d(k, ud, t, pd)) {
      const int sv = CB::save_d(k);
      if ((sv & GBDE_SAVE_BEFORE) && !exact) save(t, ud);
      exact = false;
      CB::affect_d(k, ud, t, pd, term);
      if (sv & GBDE_SAVE_AFTER) save(t, ud);
      any = true;
    }
  }
  if (any) {
#pragma unroll
    for (int c = 0; c < N; ++c) u[c] = (T)ud[c];
  }
  return any;
}

GBDE_D bool cb_crossed(double g0, double g1) {
  return (g0 < 0.0 && g1 >= 0.0) || (g0 > 0.0 && g1 <= 0.0);
}

// early_time<Alg>::v: the stepper's static constexpr bool EARLY_TIME, or false
template <class A, class = void>
struct early_time {
  static constexpr bool v = false;
};
template <class A>
struct early_time<A, decltype(void(A::EARLY_TIME))> {
  static constexpr bool v = A::EARLY_TIME;
};

// switching<Alg>::v: a composite that may change its method before an attempt
// (AutoSwitchAlg, autoswitch.cuh, specialises it); it provides
//   double choose(double dt, const T* p, int& nf)   -- the step size to attempt
//   bool stiff                                       -- the stiff method is current
//   int method() const                               -- GBDE_ALG_* of the current method
template <class A>
struct switching {
  static constexpr bool v = false;
};
// the controller constants of the stepper's current method
template <class A>
GBDE_D const CtlK& ctl_of(const A& alg, const KArgs& a) {
  if constexpr (switching<A>::v) return alg.stiff ? a.ctl_stiff : a.ctl;
  else return a.ctl;
}
template <class A>
GBDE_D int method_of(const A& alg) {
  if constexpr (switching<A>::v) return alg.method();
  else return A::ALG_ID;
}

// ------------------------------------------------------------- driver
// Alg provides:  static constexpr int ORDER (for beta defaults / init dt),
//   void init(const T* u0, const T* p, int& nf)       -- u = u0, f(u) cache
//   double attempt(double dt, const T* p, double abstol, double reltol, int& nf)
//                                                       -- returns EEst^2
//   void interp(double theta, double dt, T* out, const T* p, int& nf)
//                                                       -- dense output
//   void accept(const T* p, int& nf)                    -- u = unew, caches
//   const T* u() / unew() / f0()
template <class Alg, class M, class T, bool MIXED, class CB = NoCallback>
__device__ void integrate_all(const KArgs& a) {
  constexpr int N = M::N;
  double gprev[CB::NC > 0 ? CB::NC : 1];  // continuous conditions at the current point
  int nudge = -1;  // condition whose event ended the previous step (repeat nudge), or -1
  int nev = 0;     // event saves made by the current trajectory
  WorkSource src;
  src.init();
  Alg alg;
  T p[M::NP];
  int64_t i = -1;
  bool active = false;
  // time, end, step and first step as FP64 bit patterns (F64Bits): the loop's
  // copies and selects of them stay on the integer pipe
  F64Bits t = 0.0, tf = 0.0, dt = 0.0, dt1 = 0.0;
  const bool clamp = a.dtmax > 0.0;
  const F64Bits dtmax = a.dtmax;
  float lqold = 0.0f;  // log2(qold)
  int js = 0, nacc = 0, nrej = 0, nfev = 0;
  int64_t iters = 0;
  int ret = GBDE_RET_DEFAULT;
  const uint64_t t_start = a.timeout_ns ? global_ns() : 0;

  while (true) {
    if (!active) {
      i = src.next(a);
      if (i < 0) break;
      // ---- load the trajectory
      T u0[N];
#pragma unroll
      for (int k = 0; k < M::NP; ++k) p[k] = (T)__ldg(a.p + (size_t)i * M::NP + k);
#pragma unroll
      for (int c = 0; c < N; ++c) u0[c] = (T)__ldg(a.u0 + (size_t)i * N + c);
      t = __ldg(a.t0 + i);
      tf = __ldg(a.tf + i);
      js = 0;
      nacc = nrej = nfev = nev = 0;
      iters = 0;
      lqold = a.ctl.lqoldinit;
      dt1 = __longlong_as_double(0x7ff8000000000000ll);
      ret = GBDE_RET_DEFAULT;
      bool bad = !(tf >= t) || !isfinite(t) || !isfinite(tf);
#pragma unroll
      for (int c = 0; c < N; ++c) bad |= !isfinite((double)u0[c]);
      // save points at t0 store u0 exactly: from the FP64 input, not from its
      // copy in the working precision T (a pair holds ~48 bits, a float 24)
      if (js < a.n_save && save_time(a, i, js) <= t) {
        double u0d[N];
#pragma unroll
        for (int c = 0; c < N; ++c) u0d[c] = __ldg(a.u0 + (size_t)i * N + c);
        while (js < a.n_save && save_time(a, i, js) <= t) {
          store_state<N>(a, i, js, u0d);
          ++js;
        }
      }
      if (bad) {
        ret = GBDE_RET_INITIALFAILURE;
      } else {
        alg.init(u0, p, nfev);
        if (a.pred_dt != nullptr && a.pred_dt[i] > 0.f) {
          dt = fmin((double)a.pred_dt[i], tf - t);
        } else if (a.dt0 > 0.0 || !a.adaptive) {
          dt = a.dt0;
        } else if (a.dt_init != nullptr) {
          dt = __ldg(a.dt_init + i);  // k_init_dt: the same computation, done beforehand
          ++nfev;                     // its trial evaluation of f
        } else {
          dt = initial_dt<M, T>(alg.u(), alg.f0(), p, tf - t, Alg::ORDER, a.abstol, a.reltol,
                                nfev);
        }
        if (a.dtmax > 0.0) dt = fmin(dt, a.dtmax);
        if (!(t < tf)) ret = GBDE_RET_SUCCESS;
        else if (!(dt > 0.0)) ret = GBDE_RET_DTLESSTHANMIN;
        if constexpr (CB::NC > 0) {
          cb_conditions<CB, N, M::NP>(alg.u(), t, p, gprev);
          nudge = -1;
        }
      }
      active = true;
    }

    if (ret == GBDE_RET_DEFAULT) {
      // ---- one attempted step
      if constexpr (switching<Alg>::v) {
        if (iters > 0) {  // the method for this attempt, from the last one's estimate
          dt = alg.choose(dt, p, nfev);
          if (clamp && ord_bits(dt) > ord_bits(a.dtmax)) dt = dtmax;
        }
      }
      const double rem = tf - t;
      const bool last = ord_bits(dt * (1.0 + 1e-10)) >= ord_bits(rem);
      const F64Bits hb = last ? F64Bits(rem) : dt;
      const double h = hb;
      // The step's end if the attempt is accepted: t + h in FP64, in every
      // precision, as the FP64 oracle and the reference form it.  Steppers
      // that declare EARLY_TIME get it before the attempt, so that its FP64
      // addition overlaps the attempt's work: worth it where one warp runs
      // alone on its SM sub-partition (small ensembles), at the cost of a
      // register pair live through the attempt.
      F64Bits tnew_e = 0.0;
      if constexpr (early_time<Alg>::v) tnew_e = last ? tf : F64Bits(t + h);
      const double ms = alg.attempt(h, p, a.abstol, a.reltol, nfev);  // EEst^2
      ++iters;
      // ms <= 1 (ms >= 0; NaN rejects), compared on the integer pipe
      const bool ok = !a.adaptive || mag_bits(ms) <= 0x3FF0000000000000ull;
      if (ok) {
        // controller proposal for the next step
        double dtnew = h;
        if (a.adaptive) dtnew = h * f2d_bits(ctl_accept(ctl_of(alg, a), ms, lqold));
        F64Bits tnew;
        if constexpr (early_time<Alg>::v) tnew = tnew_e;
        else tnew = last ? tf : F64Bits(t + h);
        // continuous callbacks: crossings of the conditions in (t, tnew]
        // (for the condition that fired at t, in (t + h/100, tnew]: the
        // repeat nudge); the earliest located root is the event
        bool event = false;
        double th_e = 1.0;
        int idx_e = 0;
        if constexpr (CB::NC > 0) {
          double ga[CB::NC], gb[CB::NC];
#pragma unroll
          for (int c = 0; c < CB::NC; ++c) ga[c] = gprev[c];
          const int nudged = nudge;
          if (nudged >= 0) {
            T un[N];
            double gn[CB::NC];
            alg.interp(0.01, h, un, p, nfev);
            cb_conditions<CB, N, M::NP>(un, t + 0.01 * h, p, gn);
#pragma unroll
            for (int c = 0; c < CB::NC; ++c)
              if (c == nudged) ga[c] = gn[c];
            nudge = -1;
          }
          cb_conditions<CB, N, M::NP>(alg.unew(), tnew, p, gb);
#pragma unroll 1
          for (int ci = 0; ci < CB::NC; ++ci) {
            if (!cb_crossed(ga[ci], gb[ci])) continue;
            // Illinois regula falsi on theta in [lo, 1] for condition ci; the
            // left end keeps the sign before the crossing
            const double lo = ci == nudged ? 0.01 : 0.0;
            double a0 = lo, b0 = 1.0, fa = ga[ci], fb = gb[ci];
            int side = 0;
            for (int it = 0; it < 100; ++it) {
              if ((b0 - a0) * fabs(h) <= 8.9e-16 * fmax(fabs(t), fabs(tnew))) break;
              double m = b0 - fb * (b0 - a0) / (fb - fa);
              if (!(m > a0 && m < b0)) m = 0.5 * (a0 + b0);
              T um[N];
              alg.interp(m, h, um, p, nfev);
              double gm[CB::NC];
              cb_conditions<CB, N, M::NP>(um, t + m * h, p, gm);
              const double fm = gm[ci];
              if (fm == 0.0) {
                a0 = m;
                break;
              }
              if (cb_crossed(fa, fm)) {  // root in (a0, m]
                b0 = m;
                fb = fm;
                if (side == -1) fa *= 0.5;
                side = -1;
              } else {
                a0 = m;
                fa = fm;
                if (side == 1) fb *= 0.5;
                side = 1;
              }
            }
            if (!event || a0 < th_e) {
              th_e = a0;
              idx_e = ci;
            }
            event = true;
          }
          if (!event) {
#pragma unroll
            for (int c = 0; c < CB::NC; ++c) gprev[c] = gb[c];
          }
        }
        // saveat: dense output at every save time in (t, tnew], or up to the
        // event; `exact`: the last one stored falls on that end
        const double te = event ? t + th_e * h : (double)tnew;
        const uint64_t tnew_o = ord_bits(tnew), lim_o = ord_bits(te);
        bool exact = false;
        while (js < a.n_save) {
          const double ts = save_time(a, i, js);
          const uint64_t ts_o = ord_bits(ts);
          if (ts_o > lim_o) break;
          exact = ts_o == lim_o;
          if (!event && ts_o == tnew_o) {
            store_state<N>(a, i, js, alg.unew());
          } else {
            T tmp[N];
            alg.interp((ts - t) * rcp64(h), h, tmp, p, nfev);
            store_state<N>(a, i, js, tmp);
          }
          ++js;
        }
        // an event save: (time, state) rounded to the working precision,
        // the state the integration holds
        auto ev_save = [&](double ts, const double* ud) {
          if constexpr (CB::SAVES != 0) {
            if (a.ev_n == nullptr) return;
            if (nev < a.ev_cap) {
              const size_t o = (size_t)i * a.ev_cap + nev;
              if (a.ev_t) a.ev_t[o] = ts;
              if (a.ev_u) {
#pragma unroll
                for (int c = 0; c < N; ++c) {
                  const double v = (double)(T)ud[c];
                  if (a.out_f32) ((float*)a.ev_u)[o * N + c] = (float)v;
                  else ((double*)a.ev_u)[o * N + c] = v;
                }
              }
            }
            ++nev;
          }
        };
        if (event) {
          // move to the event, apply affect, restart the method there
          T ue[N];
          alg.interp(th_e, h, ue, p, nfev);
          const int sv = CB::save_c(idx_e);
          if ((sv & GBDE_SAVE_BEFORE) && !exact) {
            double ud[N];
#pragma unroll
            for (int c = 0; c < N; ++c) ud[c] = (double)ue[c];
            ev_save(te, ud);
          }
          bool term = cb_affect_c<CB, N, M::NP>(idx_e, ue, te, p);
          if (sv & GBDE_SAVE_AFTER) {
            double ud[N];
#pragma unroll
            for (int c = 0; c < N; ++c) ud[c] = (double)ue[c];
            ev_save(te, ud);
          }
          if constexpr (CB::ND > 0) cb_discrete<CB, N, M::NP>(ue, te, p, term, false, ev_save);
          alg.init(ue, p, nfev);
          t = te;
          nudge = idx_e;
          cb_conditions<CB, N, M::NP>(alg.u(), t, p, gprev);
          if (nacc == 0) dt1 = th_e * h;
          ++nacc;
          bool fin = true;
#pragma unroll
          for (int c = 0; c < N; ++c) fin &= val_finite(alg.u()[c]);
          if (!fin) ret = GBDE_RET_UNSTABLE;
          else if (term) ret = GBDE_RET_TERMINATED;
          dt = clamp && ord_bits(dtnew) > ord_bits(a.dtmax) ? dtmax : F64Bits(dtnew);
        } else {
          alg.accept(p, nfev);
          t = tnew;
          if (nacc == 0) dt1 = h;
          ++nacc;
          bool fin = true;
#pragma unroll
          for (int c = 0; c < N; ++c) fin &= val_finite(alg.u()[c]);
          if (!fin) ret = GBDE_RET_UNSTABLE;
          else if (last) ret = GBDE_RET_SUCCESS;
          if constexpr (CB::ND > 0) {
            T uc[N];
#pragma unroll
            for (int c = 0; c < N; ++c) uc[c] = alg.u()[c];
            bool term = false;
            if (fin && cb_discrete<CB, N, M::NP>(uc, t, p, term, exact, ev_save)) {
              alg.init(uc, p, nfev);
              if constexpr (CB::NC > 0) cb_conditions<CB, N, M::NP>(alg.u(), t, p, gprev);
              if (term) ret = GBDE_RET_TERMINATED;
            }
          }
          dt = clamp && ord_bits(dtnew) > ord_bits(a.dtmax) ? dtmax : F64Bits(dtnew);
        }
      } else {
        ++nrej;
        dt = h * f2d_bits(ctl_reject(ctl_of(alg, a), ms));
      }
      if (ret == GBDE_RET_DEFAULT) {
        if (iters >= a.maxiters) ret = GBDE_RET_MAXITERS;
        else if (a.adaptive && dt_too_small(dt, a.dtmin, t))
          ret = GBDE_RET_DTLESSTHANMIN;
        else if (a.timeout_ns && (iters & 31) == 0 && global_ns() - t_start > a.timeout_ns) {
          ret = GBDE_RET_TIMEOUT;
          atomicOr(a.flag, 1);
        }
      }
    }

    if (ret != GBDE_RET_DEFAULT) {
      // ---- finish the trajectory; save slots never reached hold NaN
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
      if (a.method_out) a.method_out[i] = method_of(alg);
      if (a.dt_first) a.dt_first[i] = dt1;
      if constexpr (CB::NC + CB::ND > 0) {
        if (a.ev_n) a.ev_n[i] = nev;
      }
      active = false;
    }
  }
}

}  // namespace gbde
