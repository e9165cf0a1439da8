// team.cuh -- trajectories that do not fit one thread: a team of W = 16
// lanes (half a warp) integrates one trajectory of a 16-state model, lane r
// owning state component r, row r of the Jacobian and row r of the W-matrix.
//
// Used for the ring of 8 Van der Pol oscillators (n = 16).  One thread per
// trajectory would need the 16x16 FP64 W-matrix (2 KB) and 7-8 stage vectors
// of 16 in registers, which spills; split over 16 lanes, each lane holds one
// row and one component of every stage.
//   * RHS: each lane evaluates its own row f_r(u) (M::f_lane), fetching the
//     few components that row depends on from the other lanes by shuffles.
//   * Error norm: a butterfly sum over the team; every lane then takes the
//     same accept/reject decision, so control flow stays team-uniform.
//   * LU with partial pivoting, distributed by rows without moving rows (the
//     rows in shared memory): at step k the team picks the unpivoted row with
//     the largest |a_k| (shuffle max on the magnitude bits + ballot), every
//     unpivoted lane reads that row and eliminates.  Triangular solves run in
//     pivot order.
//   * Saves: the 16 lanes store the 16 components of a save point as one
//     contiguous, coalesced 128-byte (FP64) or 64-byte (FP32) segment.
#pragma once
#include "rosenbrock.cuh"
#include "explicit_rk.cuh"
#include "rodas_ff.cuh"
#include "tsit5_ff.cuh"

namespace gbde {

constexpr int TEAM = 16;

// A double step length or weight as the stepper's scalar type: FP32 pairs are
// split on the integer pipe (ff_split), not by FP64 subtraction.
template <class T>
GBDE_D T team_scalar(double d) {
  if constexpr (is_ff<T>::value) return ff_split(d);
  else return (T)d;
}

struct Team {
  unsigned mask;  // the team's 16 lanes within the warp
  int lane;       // 0..15
  GBDE_D void init() {
    const int l = threadIdx.x & 31;
    lane = l & (TEAM - 1);
    mask = 0xFFFFu << (l & TEAM);
  }
  template <class T> GBDE_D T bcast(T v, int src) const { return __shfl_sync(mask, v, src, TEAM); }
  GBDE_D ff bcast(ff v, int src) const {
    return ff(__shfl_sync(mask, v.hi, src, TEAM), __shfl_sync(mask, v.lo, src, TEAM));
  }
  GBDE_D double sum(double v) const {
#pragma unroll
    for (int o = TEAM / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, TEAM);
    return v;
  }
};

// This lane's squared scaled error (the team sums them): the ratio
// err / (abstol + reltol max(|u|, |u1|)) is FP32 for FP32 state and for FP32
// pairs (on the leading parts, as the one-thread pair steppers), the square
// formed and summed in FP64; FP64 otherwise.  (GB300 issues FP64 at 1/64 of
// the FP32 rate: with the ratio in FP64 the pair Tsit5 team kernel was bound
// by its FP64 pipe.)
template <class T>
GBDE_D double lane_err2(T err, T u, T un, double abstol, double reltol) {
  if constexpr (is_ff<T>::value) {
    const float m = fmaxf(fabsf(u.hi), fabsf(un.hi));
    const double e = f2d_bits(__fdiv_rn(err.hi, fmaf((float)reltol, m, (float)abstol)));
    return e * e;
  } else if constexpr (sizeof(T) == 4) {
    const float m = fmaxf(fabsf(u), fabsf(un));
    const double e = f2d_bits(__fdiv_rn(err, fmaf((float)reltol, m, (float)abstol)));
    return e * e;
  } else {
    const double sc = abstol + reltol * fmax(fabs((double)u), fabs((double)un));
    const double e = (double)err * rcp64(sc);
    return e * e;
  }
}

// ------------------------------------------------------------- team LU
// Row-distributed LU of W (16 x 16) with partial pivoting.  Lane r's row lives
// in shared memory (team_lu_row(), 17 doubles at a stride that keeps a warp's
// row accesses conflict-free): the pivot row is read there by the 16 lanes of
// the team (one broadcast address), the elimination and the substitutions run
// as loops with run-time bounds (compact code: the fully unrolled form was the
// kernel's largest piece of code and its top stall an empty instruction
// cache), and no row sits in registers.  After factor(), row r holds the
// multipliers (L) in c < step and the U entries in c >= step, where `step` is
// the elimination step at which row r was the pivot.  piv packs the pivot lane
// of step k in bits [4k, 4k+4).  The caller writes row r of W with
// team_lu_row() before factor().
constexpr int kTeamLuStride = TEAM + 1;
constexpr int kTeamLuThreads = 128;  // team kernels run CTAs of up to 128 threads

GBDE_D double* team_lu_row() {
  __shared__ double buf[kTeamLuThreads * kTeamLuStride];
  return buf + threadIdx.x * kTeamLuStride;
}
// the row of lane `lane` of this thread's team
GBDE_D double* team_lu_row_of(int lane) {
  return team_lu_row() + (lane - (int)(threadIdx.x & (TEAM - 1))) * kTeamLuStride;
}

struct TeamLU {
  double invp;   // 1 / pivot of this lane's step
  int step;
  uint64_t piv;

  GBDE_D void factor(const Team& tm) {
    double* a = team_lu_row();
    step = -1;
    piv = 0;
    invp = 0.0;
    // Row position of this lane's row in a row-swapping LU (LAPACK getrf,
    // the reference's dense LU): swapping pivot row p with the row at
    // position k moves that row to p's old position.  Ties in |a_k| go to the
    // lowest position, as getrf's first-maximum search does, so the pivot
    // sequence is the row-swapping LU's even when entries tie.
    unsigned pos = (unsigned)tm.lane;
    __syncwarp(tm.mask);  // every lane's row is written
#pragma unroll 1
    for (int k = 0; k < TEAM; ++k) {
      const double ak = a[k];
      // pivot: unpivoted lane with the largest |a_k|, ties: lowest position
      const uint64_t key = step < 0 ? mag_bits(ak) + 1ull : 0ull;
      uint64_t m = key;
#pragma unroll
      for (int o = TEAM / 2; o > 0; o >>= 1) {
        const uint64_t x = __shfl_xor_sync(tm.mask, m, o, TEAM);
        m = x > m ? x : m;
      }
      const bool cand = key == m;
      const unsigned ppos = __reduce_min_sync(tm.mask, cand ? pos : 0xFFFFFFFFu);
      const unsigned bal =
          __ballot_sync(tm.mask, cand && pos == ppos) >> ((threadIdx.x & 31) & TEAM);
      const int p = __ffs(bal) - 1;
      if (step < 0 && pos == (unsigned)k && tm.lane != p) pos = ppos;  // swapped out
      piv |= (uint64_t)p << (4 * k);
      const double* prow = team_lu_row_of(p);
      const double inv = rcp64(prow[k]);
      bool upd = false;
      if (tm.lane == p) {
        step = k;
        invp = inv;
      } else if (step < 0) {
        const double l = ak * inv;
        a[k] = l;
        upd = l != 0.0;
      }
      // Rank-1 update of the rows with a nonzero multiplier (on the ring's W,
      // 2-3 of up to 15 per step), column-parallel: lane c updates entry c
      // of each such row.  Every updated entry gets the same fma as a
      // row-by-row update; the skipped rows would add -0 * prow[c], which
      // leaves a finite entry unchanged.
      unsigned rows = __ballot_sync(tm.mask, upd) >> ((threadIdx.x & 31) & TEAM);
      rows &= 0xFFFFu;
      __syncwarp(tm.mask);  // the multipliers are in shared memory
      const double pc = prow[tm.lane];
#pragma unroll 1
      for (; rows != 0u; rows &= rows - 1u) {
        double* ar = team_lu_row_of(__ffs(rows) - 1);
        if (tm.lane > k) ar[tm.lane] = fma(-ar[k], pc, ar[tm.lane]);
      }
      __syncwarp(tm.mask);  // step k's updates land before step k+1 reads them
    }
  }

  GBDE_D int pivot_lane(int k) const { return (int)((piv >> (4 * k)) & 15u); }

  // Solve W x = b; b is this lane's right-hand side component, the return
  // value this lane's component of x.
  GBDE_D double solve(double b, const Team& tm) const {
    const double* a = team_lu_row();
#pragma unroll 4
    for (int k = 0; k < TEAM; ++k) {  // forward: L z = P b
      const double z = tm.bcast(b, pivot_lane(k));
      if (step > k) b = fma(-a[k], z, b);
    }
    double x = 0.0;
#pragma unroll 4
    for (int k = TEAM - 1; k >= 0; --k) {  // backward: U x = z
      const double xk = tm.bcast(b * invp, pivot_lane(k));
      if (step < k) b = fma(-a[k], xk, b);
      if (tm.lane == k) x = xk;
    }
    return x;
  }
};

// ------------------------------------------------ team Rodas5 / Rodas5P
// Same transformed form as RodasAlg (rosenbrock.cuh), one component per lane.
template <class M, class T, class Tag>
struct TeamRodas {
  using K = RodasCoef<Tag>;
  static constexpr int ORDER = 4, ALG_ID = K::ALG_ID;
  static_assert(M::N == TEAM, "team kernels are for 16-state models");
  T uu, un, F0, s1, s2, s3, s4, s5, s6, s7;
  bool fresh;

  GBDE_D T u() const { return uu; }
  GBDE_D T unew() const { return un; }
  GBDE_D T f0() const { return F0; }

  GBDE_D T rhs(T y, const T* p, const Team& tm) const { return M::f_lane(tm.lane, y, p, tm); }

  GBDE_D void refresh(const T* p, const Team& tm) {
    F0 = M::f_lane(tm.lane, uu, p, tm);
    fresh = true;
  }

  GBDE_D void init(T u0, const T* p, const Team& tm, int& nf) {
    uu = u0;
    refresh(p, tm);
    ++nf;
  }

  GBDE_D double attempt(double dt, const T* p, double abstol, double reltol, const Team& tm,
                        int& nf) {
    if (!fresh) {
      refresh(p, tm);
      ++nf;
    }
    // row r of the Jacobian at uu, built afresh on every attempt: a copy
    // kept across attempts would hold 16 more registers through the stages
    TeamLU W;
    const double ih = rcp64(dt);
    const double dg = ih * (1.0 / K::g);
    {
      T Jr[TEAM];
      M::jac_lane(tm.lane, uu, p, tm, Jr);
      double* wr = team_lu_row();
#pragma unroll
      for (int c = 0; c < TEAM; ++c) wr[c] = c == tm.lane ? dg - (double)Jr[c] : -(double)Jr[c];
    }
    W.factor(tm);
    const T iht = (T)ih;  // r_i = f(y_i) + (1/h) sum_j C_ij u_j
    s1 = (T)W.solve((double)F0, tm);
    T y = uu + T(K::a21) * s1;
    s2 = (T)W.solve((double)(rhs(y, p, tm) + iht * (T(K::C21) * s1)), tm);
    y = uu + T(K::a31) * s1 + T(K::a32) * s2;
    s3 = (T)W.solve((double)(rhs(y, p, tm) + iht * (T(K::C31) * s1 + T(K::C32) * s2)), tm);
    y = uu + T(K::a41) * s1 + T(K::a42) * s2 + T(K::a43) * s3;
    s4 = (T)W.solve((double)(rhs(y, p, tm) + iht * (T(K::C41) * s1 + T(K::C42) * s2 + T(K::C43) * s3)), tm);
    y = uu + T(K::a51) * s1 + T(K::a52) * s2 + T(K::a53) * s3 + T(K::a54) * s4;
    s5 = (T)W.solve((double)(rhs(y, p, tm) + iht * (T(K::C51) * s1 + T(K::C52) * s2 + T(K::C53) * s3 + T(K::C54) * s4)), tm);
    y = uu + T(K::a61) * s1 + T(K::a62) * s2 + T(K::a63) * s3 + T(K::a64) * s4 +
        T(K::a65) * s5;
    s6 = (T)W.solve((double)(rhs(y, p, tm) + iht * (T(K::C61) * s1 + T(K::C62) * s2 + T(K::C63) * s3 + T(K::C64) * s4 + T(K::C65) * s5)), tm);
    y += s6;
    s7 = (T)W.solve((double)(rhs(y, p, tm) + iht * (T(K::C71) * s1 + T(K::C72) * s2 + T(K::C73) * s3 + T(K::C74) * s4 + T(K::C75) * s5 + T(K::C76) * s6)), tm);
    y += s7;
    const T s8 = (T)W.solve((double)(rhs(y, p, tm) + iht * (T(K::C81) * s1 + T(K::C82) * s2 + T(K::C83) * s3 + T(K::C84) * s4 + T(K::C85) * s5 + T(K::C86) * s6 + T(K::C87) * s7)), tm);
    nf += 7;
    un = y + s8;
    return tm.sum(lane_err2(s8, uu, un, abstol, reltol)) * (1.0 / TEAM);
  }

  GBDE_D T interp(double th, double) const {  // as RodasAlg::interp
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
    return uu + (T)th * (un - uu) + (e[0] * s1 + e[1] * s2 + e[2] * s3 + e[3] * s4 + e[4] * s5 +
                                     e[5] * s6 + e[6] * s7);
  }

  GBDE_D void accept() {
    uu = un;
    fresh = false;
  }
};

// ----------------------------------------------------------- team driver
// integrate_all (solver.cuh) for teams: the same controller, saves, return
// codes and deadline; every scalar decision is team-uniform.
template <class Alg, class M, class T, bool MIXED>
__device__ void integrate_team(const KArgs& a) {
  Team tm;
  tm.init();
  const int64_t team_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TEAM;
  const uint64_t t_start = a.timeout_ns ? global_ns() : 0;
  bool first = true;
  Alg alg;
  T p[M::NP];
  while (true) {
    // ---- next trajectory (team-uniform)
    int64_t i;
    if (a.queue == nullptr) {
      if (!first) break;
      i = team_id < a.N ? (a.order ? (int64_t)a.order[team_id] : team_id) : -1;
    } else {
      unsigned long long idx = 0;
      if (tm.lane == 0) idx = atomicAdd(a.queue, 1ull);
      idx = tm.bcast(idx, 0);
      i = idx < (unsigned long long)a.N ? (a.order ? (int64_t)a.order[idx] : (int64_t)idx) : -1;
    }
    first = false;
    if (i < 0) break;
#pragma unroll
    for (int k = 0; k < M::NP; ++k) p[k] = (T)__ldg(a.p + (size_t)i * M::NP + k);
    const double u0d = __ldg(a.u0 + (size_t)i * TEAM + tm.lane);
    const T u0 = (T)u0d;
    double t = __ldg(a.t0 + i);
    const double tf = __ldg(a.tf + i);
    int js = 0, nacc = 0, nrej = 0, nfev = 0;
    int64_t iters = 0;
    float lqold = a.ctl.lqoldinit;
    double dt1 = __longlong_as_double(0x7ff8000000000000ll);
    int ret = GBDE_RET_DEFAULT;
    const bool bad_lane = !isfinite((double)u0);
    const bool bad = !(tf >= t) || !isfinite(t) || !isfinite(tf) ||
                     __any_sync(tm.mask, bad_lane);
    auto store = [&](int j, double v) {  // v: FP64 value of this lane's component
      if (a.red) reduce_add(a, j, tm.lane, TEAM, v);
      if (a.u_out == nullptr) return;
      const size_t o = ((size_t)i * a.n_save + j) * TEAM + tm.lane;
      if (a.out_f32) ((float*)a.u_out)[o] = (float)v;
      else ((double*)a.u_out)[o] = v;
    };
    // save points at t0 store u0 exactly (the FP64 input, whatever T)
    while (js < a.n_save && save_time(a, i, js) <= t) store(js++, u0d);
    double dt = 0.0;
    if (bad) {
      ret = GBDE_RET_INITIALFAILURE;
    } else {
      alg.init(u0, p, tm, nfev);
      if (a.pred_dt != nullptr && a.pred_dt[i] > 0.f) {
        dt = fmin((double)a.pred_dt[i], tf - t);
      } else if (a.dt0 > 0.0 || !a.adaptive) {
        dt = a.dt0;
      } else {
        // Hairer-Wanner starting step (hw_h0 / hw_dt, controller.h)
        const double r = rcp64(a.abstol + fabs((double)alg.u()) * a.reltol);
        const double x = (double)alg.u() * r, y = (double)alg.f0() * r;
        const double s0 = tm.sum(x * x) * (1.0 / TEAM), s1 = tm.sum(y * y) * (1.0 / TEAM);
        const double h0 = hw_h0(s0, s1, tf - t);
        const T f1 = alg.rhs(alg.u() + T(h0) * alg.f0(), p, tm);
        ++nfev;
        const double z = ((double)f1 - (double)alg.f0()) * r;
        dt = hw_dt(h0, s1, tm.sum(z * z) * (1.0 / TEAM), tf - t, Alg::ORDER);
      }
      if (a.dtmax > 0.0) dt = fmin(dt, a.dtmax);
      if (!(t < tf)) ret = GBDE_RET_SUCCESS;
      else if (!(dt > 0.0)) ret = GBDE_RET_DTLESSTHANMIN;
    }
    while (ret == GBDE_RET_DEFAULT) {
      const double rem = tf - t;
      double h = dt;
      bool last = false;
      if (ord_bits(h * (1.0 + 1e-10)) >= ord_bits(rem)) {
        h = rem;
        last = true;
      }
      const double ms = alg.attempt(h, p, a.abstol, a.reltol, tm, nfev);
      ++iters;
      if (!a.adaptive || mag_bits(ms) <= 0x3FF0000000000000ull) {  // ms <= 1 (integer pipe)
        double dtnew = h;
        if (a.adaptive) dtnew = h * f2d_bits(ctl_accept(a.ctl, ms, lqold));
        const double tnew = last ? tf : t + h;  // plain FP64, as the oracle
        const uint64_t tnew_o = ord_bits(tnew);
        while (js < a.n_save) {
          const double ts = save_time(a, i, js);
          const uint64_t ts_o = ord_bits(ts);
          if (ts_o > tnew_o) break;
          store(js, (double)(ts_o == tnew_o ? alg.unew() : alg.interp((ts - t) * rcp64(h), h)));
          ++js;
        }
        alg.accept();
        t = tnew;
        if (nacc == 0) dt1 = h;
        ++nacc;
        if (__any_sync(tm.mask, !val_finite(alg.u()))) ret = GBDE_RET_UNSTABLE;
        else if (last) ret = GBDE_RET_SUCCESS;
        dt = a.dtmax > 0.0 && ord_bits(dtnew) > ord_bits(a.dtmax) ? a.dtmax : dtnew;
      } else {
        ++nrej;
        dt = h * f2d_bits(ctl_reject(a.ctl, ms));
      }
      if (ret == GBDE_RET_DEFAULT) {
        if (iters >= a.maxiters) ret = GBDE_RET_MAXITERS;
        else if (a.adaptive && dt_too_small(dt, a.dtmin, t))
          ret = GBDE_RET_DTLESSTHANMIN;
        else if (a.timeout_ns && (iters & 31) == 0) {
          // lane 0's clock decides for the team
          const int late = tm.bcast((int)(global_ns() - t_start > a.timeout_ns), 0);
          if (late) {
            ret = GBDE_RET_TIMEOUT;
            if (tm.lane == 0) atomicOr(a.flag, 1);
          }
        }
      }
    }
    for (; js < a.n_save; ++js) store(js, __longlong_as_double(0x7ff8000000000000ll));
    if (tm.lane == 0) {
      a.retcode[i] = ret;
      if (a.naccept) a.naccept[i] = nacc;
      if (a.nreject) a.nreject[i] = nrej;
      if (a.nf) a.nf[i] = nfev;
      if (a.t_end) a.t_end[i] = t;
      if (a.method_out) a.method_out[i] = Alg::ALG_ID;
      if (a.dt_first) a.dt_first[i] = dt1;
    }
  }
}

// ------------------------------------------ 8-lane Tsit5 (two components per lane)
// The explicit method needs no W-matrix, so a team of 8 lanes carries a
// trajectory of the 16-state ring with one oscillator (two components) per
// lane: 4 trajectories per warp instead of 2.  Every per-trajectory scalar
// operation of the driver (error-norm sum, step-size products, compensated
// time) runs once per team, and on GB300's narrow FP64 pipe those bound the
// 16-lane pair kernel; the right-hand side fetches two neighbours per
// oscillator instead of four per component.  Same method and arithmetic per
// component as Tsit5Alg (explicit_rk.cuh); the FP32 path keeps the compensated
// state uu + lo.
constexpr int TEAM8 = 8;

struct Team8 {
  unsigned mask;  // the team's 8 lanes within the warp
  int lane;       // 0..7: components 2 lane, 2 lane + 1
  GBDE_D void init() {
    const int l = threadIdx.x & 31;
    lane = l & (TEAM8 - 1);
    mask = 0xFFu << (l & 24);
  }
  template <class T> GBDE_D T bcast(T v, int src) const { return __shfl_sync(mask, v, src, TEAM8); }
  GBDE_D ff bcast(ff v, int src) const {
    return ff(__shfl_sync(mask, v.hi, src, TEAM8), __shfl_sync(mask, v.lo, src, TEAM8));
  }
  GBDE_D double sum(double v) const {
#pragma unroll
    for (int o = TEAM8 / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, TEAM8);
    return v;
  }
  GBDE_D float sum(float v) const {
#pragma unroll
    for (int o = TEAM8 / 2; o > 0; o >>= 1) v = xadd(v, __shfl_xor_sync(mask, v, o, TEAM8));
    return v;
  }
};

// The mean of the squared norm ratios e_c of a lane's two components over the
// team's 16, in FP32: each ratio is already an FP32 value (relative error
// ~2^-24), which the FP32 squares and sum leave at that order.  GB300 issues
// one FP64 warp instruction per ~64 cycles per SM sub-partition: the FP64
// form (2 FMAs, 3 additions, a product per attempt) was the non-stiff pair
// kernel's FP64-pipe bottleneck.  Returned as a double (integer-pipe widening).
GBDE_D double team8_mean_sq(const Team8& tm, float e0, float e1) {
  const float s = tm.sum(xfma(e1, e1, xmul(e0, e0)));
  return f2d_bits(xmul(s, 1.0f / (2 * TEAM8)));
}

// The tolerances an 8-lane stepper's attempt reads: FP64, and the FP32 values
// the pair steppers' norm ratios use (tol_f32), formed once per kernel.
struct TeamTol {
  double abstol, reltol;
  float atf, rtf;
  GBDE_D TeamTol(double a, double r) : abstol(a), reltol(r), atf(tol_f32(a)), rtf(tol_f32(r)) {}
};

template <class M, class T>
struct TeamTsit5P {
  static constexpr int ORDER = 5, ALG_ID = GBDE_ALG_TSIT5;
  static constexpr bool CMP = sizeof(T) == 4;
  static_assert(M::N == 2 * TEAM8, "8-lane teams are for 16-state models");
  T uu[2], un[2], lo[2], lon[2], k1[2], k2[2], k3[2], k4[2], k5[2], k6[2], k7[2];

  GBDE_D const T* u() const { return uu; }
  GBDE_D const T* unew() const { return un; }
  GBDE_D const T* f0() const { return k1; }

  GBDE_D T at(int c, T inc) const {
    if constexpr (CMP) return uu[c] + (lo[c] + inc);
    else return uu[c] + inc;
  }
  GBDE_D void rhs(const T* y, const T* p, const Team8& tm, T* dy) const {
    M::f_osc(tm.lane, y, p, tm, dy);
  }

  GBDE_D void init(const T* u0, const T* p, const Team8& tm, int& nf) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      uu[c] = u0[c];
      lo[c] = T(0);
    }
    rhs(uu, p, tm, k1);
    ++nf;
  }

  GBDE_D double attempt(double dt, const T* p, const TeamTol& tol, const Team8& tm,
                        int& nf) {
    using namespace tab::tsit5;
    const T h = team_scalar<T>(dt);
    T y[2];
#define GBDE_T8_STAGE(dst, expr)               \
  _Pragma("unroll") for (int c = 0; c < 2; ++c) \
    y[c] = at(c, h * (expr));                    \
  rhs(y, p, tm, dst);
    GBDE_T8_STAGE(k2, T(a21) * k1[c])
    GBDE_T8_STAGE(k3, T(a31) * k1[c] + T(a32) * k2[c])
    GBDE_T8_STAGE(k4, T(a41) * k1[c] + T(a42) * k2[c] + T(a43) * k3[c])
    GBDE_T8_STAGE(k5, T(a51) * k1[c] + T(a52) * k2[c] + T(a53) * k3[c] + T(a54) * k4[c])
    GBDE_T8_STAGE(k6, T(a61) * k1[c] + T(a62) * k2[c] + T(a63) * k3[c] + T(a64) * k4[c] +
                          T(a65) * k5[c])
#undef GBDE_T8_STAGE
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const T inc = h * (T(a71) * k1[c] + T(a72) * k2[c] + T(a73) * k3[c] + T(a74) * k4[c] +
                         T(a75) * k5[c] + T(a76) * k6[c]);
      if constexpr (CMP) two_sum_t(uu[c], lo[c] + inc, un[c], lon[c]);
      else un[c] = uu[c] + inc;
    }
    rhs(un, p, tm, k7);
    nf += 6;
    double e2 = 0.0;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const T err = h * (T(bt1) * k1[c] + T(bt2) * k2[c] + T(bt3) * k3[c] + T(bt4) * k4[c] +
                         T(bt5) * k5[c] + T(bt6) * k6[c] + T(bt7) * k7[c]);
      e2 += lane_err2(err, uu[c], un[c], tol.abstol, tol.reltol);
    }
    return tm.sum(e2) * (1.0 / M::N);
  }

  GBDE_D void interp(double th, double dt, T* out) const {
    using namespace tab::tsit5;
    const double t2 = th * th;
    const T b1 = team_scalar<T>(r11 * th * (th - r12) * (t2 - r13 * th + r14));
    const T b2 = team_scalar<T>(r21 * t2 * (t2 - r22 * th + r23));
    const T b3 = team_scalar<T>(r31 * t2 * (t2 - r32 * th + r33));
    const T b4 = team_scalar<T>(r41 * (th - r42) * (th - r43) * t2);
    const T b5 = team_scalar<T>(r51 * (th - r52) * (th - r53) * t2);
    const T b6 = team_scalar<T>(r61 * (th - r62) * (th - r63) * t2);
    const T b7 = team_scalar<T>(r71 * (th - r72) * (th - r73) * t2);
    const T h = team_scalar<T>(dt);
#pragma unroll
    for (int c = 0; c < 2; ++c)
      out[c] = at(c, h * (b1 * k1[c] + b2 * k2[c] + b3 * k3[c] + b4 * k4[c] + b5 * k5[c] +
                          b6 * k6[c] + b7 * k7[c]));
  }

  GBDE_D void accept() {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      uu[c] = un[c];
      if constexpr (CMP) lo[c] = lon[c];
      k1[c] = k7[c];
    }
  }
};

// The FP32-pair form of TeamTsit5P: a lane's two components are one paired
// FP32 register (FfVec<2>), so every stage argument, the new state, the error
// estimate and the dense output are one unnormalised accumulation of paired
// instructions over the pre-scaled stages h k_j (as Tsit5FF, tsit5_ff.cuh);
// the norm's ratios are FP32 on the leading parts, their mean square FP32
// (team8_mean_sq).
//
// The right-hand side is one out-of-line function (team8_osc_rhs) rather than
// seven inlined copies: the unrolled attempt then fits the instruction cache
// better.  Its top stall had been no_instruction; on the 16-state ring at 1M
// trajectories the non-stiff kernel went 121 -> 117.5 ms, bit for bit the same.
struct Ff2Pair {
  ff a, b;
};
template <class M>
__device__ __noinline__ Ff2Pair team8_osc_rhs(int lane, unsigned mask, ff x, ff v, ff mu, ff ka) {
  Team8 tm;
  tm.lane = lane;
  tm.mask = mask;
  const ff y[2] = {x, v}, p[2] = {mu, ka};
  ff dy[2];
  M::template f_osc_acc<FfAcc>(lane, y, p, tm, dy);
  return {dy[0], dy[1]};
}

template <class M>
struct TeamTsit5FF {
  using T = ff;
  static constexpr int ORDER = 5, ALG_ID = GBDE_ALG_TSIT5;
  static_assert(M::N == 2 * TEAM8, "8-lane teams are for 16-state models");
  ff uu[2], un[2], k1[2], k7[2];
  FfVec<2> hk[7];  // h k_j of the current attempt

  GBDE_D const ff* u() const { return uu; }
  GBDE_D const ff* unew() const { return un; }
  GBDE_D const ff* f0() const { return k1; }
  GBDE_D void rhs(const ff* y, const ff* p, const Team8& tm, ff* dy) const {
    const Ff2Pair r = team8_osc_rhs<M>(tm.lane, tm.mask, y[0], y[1], p[0], p[1]);
    dy[0] = r.a;
    dy[1] = r.b;
  }

  GBDE_D void init(const ff* u0, const ff* p, const Team8& tm, int& nf) {
    uu[0] = u0[0];
    uu[1] = u0[1];
    rhs(uu, p, tm, k1);
    ++nf;
  }

  GBDE_D double attempt(double dt, const ff* p, const TeamTol& tol, const Team8& tm,
                        int& nf) {
    using namespace tab::tsit5;
    constexpr ff A21 = ff(a21);
    constexpr ff A31 = ff(a31), A32 = ff(a32);
    constexpr ff A41 = ff(a41), A42 = ff(a42), A43 = ff(a43);
    constexpr ff A51 = ff(a51), A52 = ff(a52), A53 = ff(a53), A54 = ff(a54);
    constexpr ff A61 = ff(a61), A62 = ff(a62), A63 = ff(a63), A64 = ff(a64), A65 = ff(a65);
    constexpr ff A71 = ff(a71), A72 = ff(a72), A73 = ff(a73), A74 = ff(a74), A75 = ff(a75),
                 A76 = ff(a76);
    constexpr ff E1 = ff(bt1), E2 = ff(bt2), E3 = ff(bt3), E4 = ff(bt4), E5 = ff(bt5),
                 E6 = ff(bt6), E7 = ff(bt7);
    const ff h = ff_split(dt);
    FfVec<2> uv;
    uv.from(uu);
    ff y[2], k[2];
    FfVecAcc<2> a;
    hk[0] = ff_scale<2>(h, k1);
    a.set(uv);
    a.fma(A21, hk[0]);
    a.get(y);
    rhs(y, p, tm, k);
    hk[1] = ff_scale<2>(h, k);
    a.set(uv);
    a.fma(A31, hk[0]);
    a.fma(A32, hk[1]);
    a.get(y);
    rhs(y, p, tm, k);
    hk[2] = ff_scale<2>(h, k);
    a.set(uv);
    a.fma(A41, hk[0]);
    a.fma(A42, hk[1]);
    a.fma(A43, hk[2]);
    a.get(y);
    rhs(y, p, tm, k);
    hk[3] = ff_scale<2>(h, k);
    a.set(uv);
    a.fma(A51, hk[0]);
    a.fma(A52, hk[1]);
    a.fma(A53, hk[2]);
    a.fma(A54, hk[3]);
    a.get(y);
    rhs(y, p, tm, k);
    hk[4] = ff_scale<2>(h, k);
    a.set(uv);
    a.fma(A61, hk[0]);
    a.fma(A62, hk[1]);
    a.fma(A63, hk[2]);
    a.fma(A64, hk[3]);
    a.fma(A65, hk[4]);
    a.get(y);
    rhs(y, p, tm, k);
    hk[5] = ff_scale<2>(h, k);
    a.set(uv);
    a.fma(A71, hk[0]);
    a.fma(A72, hk[1]);
    a.fma(A73, hk[2]);
    a.fma(A74, hk[3]);
    a.fma(A75, hk[4]);
    a.fma(A76, hk[5]);
    a.get(un);
    rhs(un, p, tm, k7);
    hk[6] = ff_scale<2>(h, k7);
    nf += 6;
    ff err[2];
    a.zero();
    a.fma(E1, hk[0]);
    a.fma(E2, hk[1]);
    a.fma(E3, hk[2]);
    a.fma(E4, hk[3]);
    a.fma(E5, hk[4]);
    a.fma(E6, hk[5]);
    a.fma(E7, hk[6]);
    a.get(err);
    const float atf = tol.atf, rtf = tol.rtf;
    float e[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const float m = fmaxf(fabsf(uu[c].hi), fabsf(un[c].hi));
      e[c] = norm_ratio(err[c].hi, fmaf(rtf, m, atf));
    }
    return team8_mean_sq(tm, e[0], e[1]);
  }

  // Tsit5's interpolation polynomials in pair arithmetic (as Tsit5FF::interp)
  GBDE_D void interp(double th, double, ff* out) const {
    using namespace tab::tsit5;
    constexpr ff R11 = ff(r11), R12 = ff(r12), R13 = ff(r13), R14 = ff(r14);
    constexpr ff R21 = ff(r21), R22 = ff(r22), R23 = ff(r23);
    constexpr ff R31 = ff(r31), R32 = ff(r32), R33 = ff(r33);
    constexpr ff R41 = ff(r41), R42 = ff(r42), R43 = ff(r43);
    constexpr ff R51 = ff(r51), R52 = ff(r52), R53 = ff(r53);
    constexpr ff R61 = ff(r61), R62 = ff(r62), R63 = ff(r63);
    constexpr ff R71 = ff(r71), R72 = ff(r72), R73 = ff(r73);
    const ff t = ff_split(th), t2 = t * t;
    FfVec<2> uv;
    uv.from(uu);
    FfVecAcc<2> a;
    a.set(uv);
    a.fma(R11 * t * (t - R12) * (t2 - R13 * t + R14), hk[0]);
    a.fma(R21 * t2 * (t2 - R22 * t + R23), hk[1]);
    a.fma(R31 * t2 * (t2 - R32 * t + R33), hk[2]);
    a.fma(R41 * (t - R42) * (t - R43) * t2, hk[3]);
    a.fma(R51 * (t - R52) * (t - R53) * t2, hk[4]);
    a.fma(R61 * (t - R62) * (t - R63) * t2, hk[5]);
    a.fma(R71 * (t - R72) * (t - R73) * t2, hk[6]);
    a.get(out);
  }

  GBDE_D void accept() {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      uu[c] = un[c];
      k1[c] = k7[c];
    }
  }
};

// ----------------------------------- 8-lane Rodas (one oscillator per lane)
// The 16-state ring's stiff trajectories on teams of 8 lanes: lane l owns
// oscillator l (components 2l, 2l + 1 of the state and of every stage, rows
// 2l and 2l + 1 of W), so a warp carries 4 trajectories and the pair
// arithmetic of a lane's two components runs on paired FP32 instructions
// (FfAcc2, FfVec<2>).
// CTA size of the 8-lane pair Rodas kernel, which its shared stage buffer is
// sized for: 12 teams, 10.8 KB, 6 CTAs per SM (96 registers)
constexpr int kTeam8Threads = 96;

// Solves with the ring's W = dg I - J on an 8-lane team (lane l: oscillator
// l, unknowns x_l = 2l and v_l = 2l + 1).  W's nonzeros (VdpRing8::w_osc_nz):
//   row 2l:      dg x_l - v_l                                   = b_2l
//   row 2l + 1:  w10_l x_l + w11_l v_l - ka (x_{l-1} + x_{l+1}) = b_2l+1
// v_l enters no other row, so row 2l gives it exactly, v_l = dg x_l - b_2l
// (its pivot is -1: no choice to make), and substituting it leaves the Schur
// complement on the positions, an 8 x 8 cyclic tridiagonal system
//   A x = c,  A_ll = w10_l + w11_l dg,  A_l,l+-1 = -ka,  c_l = b_2l+1 + w11_l b_2l.
// A^-1 is formed once per attempt by Gauss-Jordan elimination with partial
// pivoting in FP32, lane l holding row l of [A | I] in registers (the pivot
// of column k: the open row with the largest |a_k|, ties to the lowest lane);
// a solve is then the product of A^-1 with c (every c_m broadcast), and v
// from its formula.  A's diagonal, c and v are formed in pairs (each may
// cancel) and rounded once.  The callers refine every solve once against W
// in pairs.
struct RingSchur8 {
  float e[TEAM8];  // row l of A^-1 on lane l
  ff w11, dg;
  float w11f, dgf;

  GBDE_D void build(ff dg_, ff w10, ff w11_, ff ka, const Team8& tm) {
    dg = dg_;
    w11 = w11_;
    w11f = (float)w11_;
    dgf = (float)dg_;
    const int l = tm.lane;
    const float ad = (float)(w10 + w11 * dg), nk = -(float)ka;
    float a[TEAM8];
#pragma unroll
    for (int m = 0; m < TEAM8; ++m) {
      a[m] = m == l ? ad : (m == ((l + 1) & (TEAM8 - 1)) || m == ((l + TEAM8 - 1) & (TEAM8 - 1)))
                               ? nk
                               : 0.0f;
      e[m] = m == l ? 1.0f : 0.0f;
    }
    bool open = true;
    unsigned piv = 0;  // pivot lane of column k in bits [3k, 3k+3)
#pragma unroll
    for (int k = 0; k < TEAM8; ++k) {
      // pivot: the open row of largest |a_k| (its bit pattern with the 3 low
      // mantissa bits dropped), ties to the lowest lane; the key's low bits
      // carry the lane, so one 32-bit max over the team decides
      unsigned m = open ? ((((__float_as_uint(a[k]) & 0x7fffffffu) >> 3) + 1u) << 3) |
                              (unsigned)(TEAM8 - 1 - l)
                        : 0u;
#pragma unroll
      for (int o = TEAM8 / 2; o > 0; o >>= 1) m = umax(m, __shfl_xor_sync(tm.mask, m, o, TEAM8));
      const int p = TEAM8 - 1 - (int)(m & (TEAM8 - 1));
      piv |= (unsigned)p << (3 * k);
      const bool me = l == p;
      // the fast reciprocal (within 1 ulp): the inverse is refined against
      // in pairs anyway, and the IEEE-rounded one sat on the pivot chain
      const float inv = __fdividef(1.0f, tm.bcast(a[k], p));
      const float f = me ? 0.0f : xmul(a[k], inv);  // this row's multiplier
#pragma unroll
      for (int c = k + 1; c < TEAM8; ++c) {
        const float v = tm.bcast(a[c], p);
        a[c] = me ? xmul(v, inv) : xfma(-f, v, a[c]);
      }
#pragma unroll
      for (int c = 0; c < TEAM8; ++c) {
        const float v = tm.bcast(e[c], p);
        e[c] = me ? xmul(v, inv) : xfma(-f, v, e[c]);
      }
      if (me) open = false;
    }
    // lane l takes row l of A^-1 (held by the lane that pivoted column l),
    // so that every product below lands on its own lane
    const int src = (int)((piv >> (3 * l)) & (TEAM8 - 1));
#pragma unroll
    for (int m = 0; m < TEAM8; ++m) e[m] = tm.bcast(e[m], src);
  }

  // x_l = (A^-1 c)_l for this lane's c_l
  GBDE_D float apply(float c, const Team8& tm) const {
    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
    for (int m = 0; m < TEAM8; m += 2) {
      s0 = xfma(e[m], tm.bcast(c, m), s0);
      s1 = xfma(e[m + 1], tm.bcast(c, m + 1), s1);
    }
    return xadd(s0, s1);
  }
  // (x_l, v_l) in FP32 from this lane's b_2l, b_2l+1 (b[0], b[1], pairs): c
  // formed in pairs (it may cancel); v in FP32 -- its rounding is exactly
  // what the refinement's residual then sees in row 2l, and corrects
  GBDE_D void solve(const ff* b, float* xv, const Team8& tm) const {
    const float x = apply((float)(b[1] + w11 * b[0]), tm);
    xv[0] = x;
    xv[1] = xfma(dgf, x, -b[0].hi);
  }
  // the same from FP32 b, all in FP32: for a refinement's correction, whose
  // relative error then only scales the (already small) correction
  GBDE_D void solve32(const float* b, float* xv, const Team8& tm) const {
    const float x = apply(xfma(w11f, b[0], b[1]), tm);
    xv[0] = x;
    xv[1] = xfma(dgf, x, -b[0]);
  }
};

// Rodas5 / Rodas5P in FP32 pairs on 8-lane teams (the method of RodasFF,
// rodas_ff.cuh, for a lane's two components): Jacobian rows and W's nonzeros
// in pairs; each stage's solve through W's Schur complement on the positions
// (RingSchur8, its 8 x 8 inverse in FP32) refined once against W in pairs;
// stage sums and dense output on paired FP32 instructions; the norm's ratios
// and their mean square FP32 (team8_mean_sq).
template <class M, class Tag>
struct TeamRodasFF8 {
  using K = RodasCoef<Tag>;
  using T = ff;
  static constexpr int ORDER = 4, ALG_ID = K::ALG_ID;
  static_assert(M::N == 2 * TEAM8, "8-lane teams are for 16-state models");
  ff uu[2], un[2];
  ff F0[2];  // f(u0): read only by the Hairer-Wanner starting step after init()
  bool fresh;  // uu's f evaluation already counted

  GBDE_D const ff* u() const { return uu; }
  GBDE_D const ff* unew() const { return un; }
  GBDE_D const ff* f0() const { return F0; }
  GBDE_D void rhs(const ff* y, const ff* p, const Team8& tm, ff* dy) const {
    M::template f_osc_acc<FfAcc>(tm.lane, y, p, tm, dy);
  }

  // stages u_1..u_7 of this lane's two components: one 16-byte (hi pair, lo
  // pair) slot per stage at stride kTeam8Threads
  GBDE_D static ulonglong2* stages() {
    __shared__ ulonglong2 buf[7 * kTeam8Threads];
    return buf + threadIdx.x;
  }
  GBDE_D static FfVec<2> ld(int j) {
    const ulonglong2 x = stages()[j * kTeam8Threads];
    FfVec<2> v;
    v.h[0].v = x.x;
    v.l[0].v = x.y;
    return v;
  }
  GBDE_D static void st(int j, const ff* x) {
    stages()[j * kTeam8Threads] =
        make_ulonglong2(f2_pack(x[0].hi, x[1].hi).v, f2_pack(x[0].lo, x[1].lo).v);
  }

  GBDE_D void init(const ff* u0, const ff* p, const Team8& tm, int& nf) {
    uu[0] = u0[0];
    uu[1] = u0[1];
    rhs(uu, p, tm, F0);
    ++nf;
    fresh = true;
  }

  GBDE_D double attempt(double dt, const ff* p, const TeamTol& tol, const Team8& tm,
                        int& nf) {
    if (!fresh) {
      ++nf;
      fresh = true;
    }
    const double ih = rcp64(dt);
    // W = I/(h gamma) - J(uu): the nonzeros of rows 2l, 2l + 1 in pairs (for
    // the residuals), the rows rounded to FP32 for the LU
    const ff dg = ff_split(ih * (1.0 / K::g));
    ff w10, w11;
    M::w_osc_nz(uu, p, dg, w10, w11);
    RingSchur8 L;
    L.build(dg, w10, w11, p[1], tm);
    const ff iht = ff_split(ih);
    const RodasFfTab& tb = c_rodas_ff[RodasFfIdx<Tag>::v];
    FfVec<2> uv;
    uv.from(uu);
    ff y[2], s[2];
#pragma unroll 1
    for (int i = 0; i < 8; ++i) {
      // stage argument: u0 for stage 1, a fresh combination for stages 2-6;
      // for 7 and 8 the previous argument plus the previous stage
      FfVecAcc<2> ya, ca;
      const bool fresh_arg = i <= 5;
      if (fresh_arg) {
        ya.set(uv);
      } else {
        FfVec<2> yv;
        yv.from(y);
        ya.set(yv);
      }
      ca.zero();
#pragma unroll 1
      for (int j = 0; j < i; ++j) {
        const ff cij = tb.rc[i][j];
        const ff aij = tb.ra[fresh_arg ? i : 0][fresh_arg ? j : 0];
        const FfVec<2> sj = ld(j);
        if (fresh_arg) ya.fma(aij, sj);
        else if (j == i - 1) ya.add(sj);
        ca.fma(cij, sj);
      }
      ff fy[2], r[2];
      ya.get(y);
      rhs(y, p, tm, fy);
      if (i > 0) {
        ff cs[2];
        ca.get(cs);
        FfVec<2> fv, cv;
        fv.from(fy);
        cv.from(cs);
        FfVecAcc<2> ra;
        ra.set(fv);
        ra.fma(iht, cv);
        ra.get(r);
      } else {
        r[0] = fy[0];
        r[1] = fy[1];
      }
      ff x[2];
      {
        // W x = r: an FP32 solve (RingSchur8) and one refinement against W in
        // pairs, x = x0 + d with W d ~ r - W x0 (residual in pairs, its
        // correction solved in FP32).  W = I/(h gamma) - J is well conditioned
        // here, so the refined error is about (cond 2^-24)^2 of |x|, far below
        // the tolerances.
        float x0[2], d[2];
        L.solve(r, x0, tm);
        ff res[2];
        M::template w_osc_residual<FfAcc>(tm.lane, dg, w10, w11, p[1], r, x0, tm, res);
        const float rf[2] = {res[0].hi, res[1].hi};
        L.solve32(rf, d, tm);
        x[0] = ff(x0[0], 0.0f) + ff(d[0], 0.0f);
        x[1] = ff(x0[1], 0.0f) + ff(d[1], 0.0f);
      }
      if (i < 7) {
        st(i, x);
      } else {
        s[0] = x[0];
        s[1] = x[1];
      }
    }
    nf += 7;
    // y1 = U_7 + u_8; error estimate u_8 (ratios FP32 on the leading parts,
    // their mean square in FP32)
    const float atf = tol.atf, rtf = tol.rtf;
    float e[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      FfAcc a;
      a.set(y[c]);
      a.add(s[c]);
      un[c] = a.get();
      const float m = fmaxf(fabsf(uu[c].hi), fabsf(un[c].hi));
      e[c] = norm_ratio(s[c].hi, fmaf(rtf, m, atf));
    }
    return team8_mean_sq(tm, e[0], e[1]);
  }

  // dense output as RodasFF::interp for the lane's two components
  GBDE_D void interp(double th, double, ff* out) const {
    const RodasFfTab& tb = c_rodas_ff[RodasFfIdx<Tag>::v];
    const ff tt = ff_split(th);
    const ff w = tt * (ff(1.0f, 0.0f) - tt);
    ff du[2];
    du[0] = un[0] - uu[0];
    du[1] = un[1] - uu[1];
    FfVec<2> uv, dv;
    uv.from(uu);
    dv.from(du);
    FfVecAcc<2> a;
    a.set(uv);
    a.fma(tt, dv);
#pragma unroll 1
    for (int j = 0; j < 7; ++j) {
      FfAcc q;
      q.set(tb.h3[j]);
      q.fma(tt, tb.h4[j]);
      const ff q3 = q.get();
      q.set(tb.h2[j]);
      q.fma(tt, q3);
      a.fma(w * q.get(), ld(j));
    }
    a.get(out);
  }

  GBDE_D void accept() {
    uu[0] = un[0];
    uu[1] = un[1];
    fresh = false;
  }
};

// integrate_team for 8-lane teams with two components per lane: the same
// controller, saves, return codes and deadline.  One flat loop: a team whose
// trajectory has ended writes its results and takes the next one inside the
// loop body, then rejoins the other teams of its warp at the attempt, so the
// warp's four teams step together instead of waiting, trajectory by
// trajectory, for the one with the most steps.
template <class Alg, class M, class T, bool MIXED>
__device__ void integrate_team8(const KArgs& a) {
  Team8 tm;
  tm.init();
  const int64_t team_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TEAM8;
  const TeamTol tol(a.abstol, a.reltol);
  const uint64_t t_start = a.timeout_ns ? global_ns() : 0;
  bool first = true;
  Alg alg;
  T p[M::NP];
  const int c0 = 2 * tm.lane;  // this lane's first component
  int64_t i = -1;              // the team's trajectory (-1: none yet)
  // time, end, step and first step as FP64 bit patterns: the loop's copies and
  // selects of them stay on the integer pipe (GB300's FP64 pipe is narrow);
  // the arithmetic reads them through D()
  uint64_t t = 0, tf = 0, dt = 0, dt1 = 0;
  auto D = [](uint64_t b) { return __longlong_as_double((long long)b); };
  auto B = [](double x) { return (uint64_t)__double_as_longlong(x); };
  const bool clamp = a.dtmax > 0.0;
  const uint64_t dtmax_b = B(a.dtmax);
  int js = 0, nacc = 0, nrej = 0, nfev = 0;
  int64_t iters = 0;
  float lqold = 0.0f;
  int ret = GBDE_RET_SUCCESS;  // anything but DEFAULT: take a trajectory
  // FP64 values of this lane's components (the inputs at t0, NaN); store_t
  // the stepper's own: the FP32 output takes a pair's hi + lo in one FP32
  // addition (rounded once, no conversions on the FP64 pipe, where a save
  // made by one team of the warp costs four times its lanes)
  auto store_t = [&](int j, const T& v0, const T& v1) {
    if (a.red) {
      reduce_add(a, j, c0, M::N, (double)v0);
      reduce_add(a, j, c0 + 1, M::N, (double)v1);
    }
    if (a.u_out == nullptr) return;
    const size_t o = ((size_t)i * a.n_save + j) * M::N + c0;
    if (a.out_f32) {
      ((float*)a.u_out)[o] = val_f32(v0);
      ((float*)a.u_out)[o + 1] = val_f32(v1);
    } else {
      ((double*)a.u_out)[o] = (double)v0;
      ((double*)a.u_out)[o + 1] = (double)v1;
    }
  };
  auto store = [&](int j, double v0, double v1) {
    if (a.red) {
      reduce_add(a, j, c0, M::N, v0);
      reduce_add(a, j, c0 + 1, M::N, v1);
    }
    if (a.u_out == nullptr) return;
    const size_t o = ((size_t)i * a.n_save + j) * M::N + c0;
    if (a.out_f32) {
      ((float*)a.u_out)[o] = (float)v0;
      ((float*)a.u_out)[o + 1] = (float)v1;
    } else {
      ((double*)a.u_out)[o] = v0;
      ((double*)a.u_out)[o + 1] = v1;
    }
  };
  while (true) {
    if (ret != GBDE_RET_DEFAULT) {
      // ---- finish the trajectory; save slots never reached hold NaN
      if (i >= 0) {
        const double nanv = __longlong_as_double(0x7ff8000000000000ll);
        for (; js < a.n_save; ++js) store(js, nanv, nanv);
        if (tm.lane == 0) {
          a.retcode[i] = ret;
          if (a.naccept) a.naccept[i] = nacc;
          if (a.nreject) a.nreject[i] = nrej;
          if (a.nf) a.nf[i] = nfev;
          if (a.t_end) a.t_end[i] = D(t);
          if (a.method_out) a.method_out[i] = Alg::ALG_ID;
          if (a.dt_first) a.dt_first[i] = D(dt1);
        }
      }
      // ---- next trajectory (team-uniform)
      if (a.queue == nullptr) {
        i = first && team_id < a.N ? (a.order ? (int64_t)a.order[team_id] : team_id) : -1;
      } else {
        unsigned long long idx = 0;
        if (tm.lane == 0) idx = atomicAdd(a.queue, 1ull);
        idx = tm.bcast(idx, 0);
        i = idx < (unsigned long long)a.N ? (a.order ? (int64_t)a.order[idx] : (int64_t)idx) : -1;
      }
      first = false;
      if (i < 0) break;
#pragma unroll
      for (int k = 0; k < M::NP; ++k) p[k] = (T)__ldg(a.p + (size_t)i * M::NP + k);
      // scalar loads and stores: the caller's arrays need only element alignment
      const double u0x = __ldg(a.u0 + (size_t)i * M::N + c0);
      const double u0y = __ldg(a.u0 + (size_t)i * M::N + c0 + 1);
      const T u0[2] = {(T)u0x, (T)u0y};
      const double t0d = __ldg(a.t0 + i), tfd = __ldg(a.tf + i);
      t = B(t0d);
      tf = B(tfd);
      js = nacc = nrej = nfev = 0;
      iters = 0;
      lqold = a.ctl.lqoldinit;
      dt1 = 0x7ff8000000000000ull;  // NaN
      ret = GBDE_RET_DEFAULT;
      const bool bad_lane = !isfinite(u0x) || !isfinite(u0y);
      const bool bad = !(tfd >= t0d) || !isfinite(t0d) || !isfinite(tfd) ||
                       __any_sync(tm.mask, bad_lane);
      // save points at t0 store u0 exactly (the FP64 input, whatever T)
      while (js < a.n_save && save_time(a, i, js) <= t0d) store(js++, u0x, u0y);
      double dtd = 0.0;
      if (bad) {
        ret = GBDE_RET_INITIALFAILURE;
      } else {
        alg.init(u0, p, tm, nfev);
        if (a.pred_dt != nullptr && a.pred_dt[i] > 0.f) {
          dtd = fmin((double)a.pred_dt[i], tfd - t0d);
        } else if (a.dt0 > 0.0 || !a.adaptive) {
          dtd = a.dt0;
        } else {
          // Hairer-Wanner starting step (hw_h0 / hw_dt, controller.h)
          double r[2], s0 = 0.0, s1 = 0.0;
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            r[c] = rcp64(a.abstol + fabs((double)alg.u()[c]) * a.reltol);
            const double x = (double)alg.u()[c] * r[c], y = (double)alg.f0()[c] * r[c];
            s0 += x * x;
            s1 += y * y;
          }
          s0 = tm.sum(s0) * (1.0 / M::N);
          s1 = tm.sum(s1) * (1.0 / M::N);
          const double h0 = hw_h0(s0, s1, tfd - t0d);
          T y[2], f1[2];
#pragma unroll
          for (int c = 0; c < 2; ++c) y[c] = alg.u()[c] + T(h0) * alg.f0()[c];
          alg.rhs(y, p, tm, f1);
          ++nfev;
          double s2 = 0.0;
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            const double z = ((double)f1[c] - (double)alg.f0()[c]) * r[c];
            s2 += z * z;
          }
          dtd = hw_dt(h0, s1, tm.sum(s2) * (1.0 / M::N), tfd - t0d, Alg::ORDER);
        }
        if (clamp) dtd = fmin(dtd, a.dtmax);
        if (!(t0d < tfd)) ret = GBDE_RET_SUCCESS;
        else if (!(dtd > 0.0)) ret = GBDE_RET_DTLESSTHANMIN;
      }
      dt = B(dtd);
      if (ret != GBDE_RET_DEFAULT) continue;  // ended before any step
    }
    // ---- one attempted step
    const double rem = D(tf) - D(t);
    const bool last = ord_bits(D(dt) * (1.0 + 1e-10)) >= ord_bits(rem);
    const uint64_t hb = last ? B(rem) : dt;
    const double h = D(hb);
    const double ms = alg.attempt(h, p, tol, tm, nfev);
    ++iters;
    if (!a.adaptive || mag_bits(ms) <= 0x3FF0000000000000ull) {  // ms <= 1 (integer pipe)
      double dtnew = h;
      if (a.adaptive) dtnew = h * f2d_bits(ctl_accept(a.ctl, ms, lqold));
      const uint64_t tnew = last ? tf : B(D(t) + h);  // plain FP64, as the oracle
      const uint64_t tnew_o = ord_bits(D(tnew));
      while (js < a.n_save) {
        const double ts = save_time(a, i, js);
        const uint64_t ts_o = ord_bits(ts);
        if (ts_o > tnew_o) break;
        if (ts_o == tnew_o) {
          store_t(js, alg.unew()[0], alg.unew()[1]);
        } else {
          T v[2];
          alg.interp((ts - D(t)) * rcp64(h), h, v);
          store_t(js, v[0], v[1]);
        }
        ++js;
      }
      alg.accept();
      t = tnew;
      if (nacc == 0) dt1 = hb;
      ++nacc;
      if (__any_sync(tm.mask, !val_finite(alg.u()[0]) || !val_finite(alg.u()[1])))
        ret = GBDE_RET_UNSTABLE;
      else if (last) ret = GBDE_RET_SUCCESS;
      dt = clamp && ord_bits(dtnew) > ord_bits(a.dtmax) ? dtmax_b : B(dtnew);
    } else {
      ++nrej;
      dt = B(h * f2d_bits(ctl_reject(a.ctl, ms)));
    }
    if (ret == GBDE_RET_DEFAULT) {
      if (iters >= a.maxiters) ret = GBDE_RET_MAXITERS;
      else if (a.adaptive && dt_too_small(D(dt), a.dtmin, D(t)))
        ret = GBDE_RET_DTLESSTHANMIN;
      else if (a.timeout_ns && (iters & 31) == 0) {
        // lane 0's clock decides for the team
        const int late = tm.bcast((int)(global_ns() - t_start > a.timeout_ns), 0);
        if (late) {
          ret = GBDE_RET_TIMEOUT;
          if (tm.lane == 0) atomicOr(a.flag, 1);
        }
      }
    }
  }
}

}  // namespace gbde
