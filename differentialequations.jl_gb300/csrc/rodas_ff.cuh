// rodas_ff.cuh -- Rodas5 / Rodas5P in FP32 pairs (the F32X2 precision) with a
// compact step body.
//
// Same method as RodasAlg (rosenbrock.cuh; OrdinaryDiffEq's Rodas5P, test/qa/qa.jl:97,
// the stiff method of test/core.jl:38-49): the transformed 8-stage form
//   (I/(h gamma) - J) u_i = f(y0 + sum_{j<i} a_ij u_j) + (1/h) sum_{j<i} C_ij u_j,
// y1 = U_7 + u_8, error estimate u_8.  What differs is where each operation runs:
//
//  * state, stages, right-hand sides and the stage combinations are FP32 pairs
//    (ff.cuh, ~48 significant bits) on the FP32 pipe, which GB300 runs at 61x its
//    FP64 rate;
//  * the Jacobian, the W-matrix and its partial-pivot LU are FP64, as is the error
//    norm's accumulation; the LU factors reach the pair solves through an
//    integer-pipe split (ff_split), not through FP64 conversions;
//  * the stage loop is not unrolled and the transformed stages live in shared
//    memory (7 x N pairs per thread), so the body stays small enough for the
//    instruction cache -- a fully unrolled pair body is several times larger than
//    its FP64 counterpart;
//  * sums of products accumulate unnormalised (FfAcc: one TwoSum per term, one
//    renormalisation per sum) instead of renormalising after every operation.
// The FP64 pipe then carries about a quarter of the instructions per attempted
// step that the FP64 stepper issues (Robertson, n = 3).
#pragma once
#include "ff_vec.cuh"
#include "rosenbrock.cuh"

namespace gbde {

// The FP64 LU factors as pairs, negated so that the substitutions are sums of
// products: nL (strictly lower), nU (strictly upper), inv (reciprocal pivots).
// The row swaps recorded in piv are applied to the right-hand side first (the
// factorisation swaps whole rows: P W = L U).
template <int N>
struct FfLU {
  ff nL[N][N], nU[N][N], inv[N];
  int piv[N];
  GBDE_D void from(const SmallLU<N>& W) {
#pragma unroll
    for (int r = 0; r < N; ++r) {
#pragma unroll
      for (int c = 0; c < N; ++c) {
        if (c < r) nL[r][c] = ff_split(-W.A[r][c]);
        if (c > r) nU[r][c] = ff_split(-W.A[r][c]);
      }
      inv[r] = ff_split(W.inv[r]);
      piv[r] = W.piv[r];
    }
  }
  GBDE_D void solve(ff* b) const {
#pragma unroll
    for (int k = 0; k < N; ++k) {
#pragma unroll
      for (int r = k + 1; r < N; ++r) {
        const bool sw = piv[k] == r;
        const ff x = b[k], y = b[r];
        b[k] = sw ? y : x;
        b[r] = sw ? x : y;
      }
    }
#pragma unroll
    for (int r = 1; r < N; ++r) {
      FfAcc acc;
      acc.set(b[r]);
#pragma unroll
      for (int k = 0; k < r; ++k) acc.fma(nL[r][k], b[k]);
      b[r] = acc.get();
    }
#pragma unroll
    for (int r = N - 1; r >= 0; --r) {
      FfAcc acc;
      acc.set(b[r]);
#pragma unroll
      for (int c = r + 1; c < N; ++c) acc.fma(nU[r][c], b[c]);
      b[r] = acc.get() * inv[r];
    }
  }
};

// Stage coefficients as pairs, indexed by the (warp-uniform) stage counters:
// ra[i][j] = a_{i+1,j+1} for the stages whose argument is a fresh sum (i <= 5),
// rc[i][j] = C_{i+1,j+1}.
// h2, h3, h4: the dense-output coefficients H2_j, H3_j, H4_j.
struct RodasFfTab {
  ff ra[6][5];
  ff rc[8][7];
  ff h2[7], h3[7], h4[7];
};

template <class K>
constexpr RodasFfTab rodas_ff_tab() {
  return RodasFfTab{
      {{ff(0.0), ff(0.0), ff(0.0), ff(0.0), ff(0.0)},
       {ff(K::a21), ff(0.0), ff(0.0), ff(0.0), ff(0.0)},
       {ff(K::a31), ff(K::a32), ff(0.0), ff(0.0), ff(0.0)},
       {ff(K::a41), ff(K::a42), ff(K::a43), ff(0.0), ff(0.0)},
       {ff(K::a51), ff(K::a52), ff(K::a53), ff(K::a54), ff(0.0)},
       {ff(K::a61), ff(K::a62), ff(K::a63), ff(K::a64), ff(K::a65)}},
      {{ff(0.0), ff(0.0), ff(0.0), ff(0.0), ff(0.0), ff(0.0), ff(0.0)},
       {ff(K::C21), ff(0.0), ff(0.0), ff(0.0), ff(0.0), ff(0.0), ff(0.0)},
       {ff(K::C31), ff(K::C32), ff(0.0), ff(0.0), ff(0.0), ff(0.0), ff(0.0)},
       {ff(K::C41), ff(K::C42), ff(K::C43), ff(0.0), ff(0.0), ff(0.0), ff(0.0)},
       {ff(K::C51), ff(K::C52), ff(K::C53), ff(K::C54), ff(0.0), ff(0.0), ff(0.0)},
       {ff(K::C61), ff(K::C62), ff(K::C63), ff(K::C64), ff(K::C65), ff(0.0), ff(0.0)},
       {ff(K::C71), ff(K::C72), ff(K::C73), ff(K::C74), ff(K::C75), ff(K::C76), ff(0.0)},
       {ff(K::C81), ff(K::C82), ff(K::C83), ff(K::C84), ff(K::C85), ff(K::C86), ff(K::C87)}},
      {ff(K::H2[0]), ff(K::H2[1]), ff(K::H2[2]), ff(K::H2[3]), ff(K::H2[4]), ff(K::H2[5]), ff(K::H2[6])},
      {ff(K::H3[0]), ff(K::H3[1]), ff(K::H3[2]), ff(K::H3[3]), ff(K::H3[4]), ff(K::H3[5]), ff(K::H3[6])},
      {ff(K::H4[0]), ff(K::H4[1]), ff(K::H4[2]), ff(K::H4[3]), ff(K::H4[4]), ff(K::H4[5]), ff(K::H4[6])}};
}

static __constant__ RodasFfTab c_rodas_ff[2] = {rodas_ff_tab<RodasCoef<Rodas5Tag>>(),
                                                rodas_ff_tab<RodasCoef<Rodas5PTag>>()};

template <class Tag> struct RodasFfIdx;
template <> struct RodasFfIdx<Rodas5Tag> { static constexpr int v = 0; };
template <> struct RodasFfIdx<Rodas5PTag> { static constexpr int v = 1; };

// Threads per CTA the stage buffer is sized for (the step kernels launch at
// most 128: __launch_bounds__(128)).
constexpr int kFfStageThreads = 128;

template <class M, class Tag>
struct RodasFF {
  using K = RodasCoef<Tag>;
  using T = ff;
  static constexpr int ORDER = 4, ALG_ID = K::ALG_ID, N = M::N;
  ff uu[N], un[N];
  ff F0[N];  // f(u0): read only by the Hairer-Wanner starting step after init()
  double pd[M::NP];
  bool fresh;  // uu's f evaluation already counted

  GBDE_D const ff* u() const { return uu; }
  GBDE_D const ff* unew() const { return un; }
  GBDE_D const ff* f0() const { return F0; }

  // Transformed stages u_1..u_7 of the current step in shared memory, per
  // thread at stride kFfStageThreads: for each component pair (2q, 2q+1) one
  // 16-byte (hi pair, lo pair) slot -- loaded straight into paired registers --
  // and for an odd last component one 8-byte (hi, lo) slot.
  static constexpr int Q = N / 2;
  GBDE_D static ulonglong2* pair_stages() {
    __shared__ ulonglong2 buf[7 * (Q > 0 ? Q : 1) * kFfStageThreads];
    return buf + threadIdx.x;
  }
  GBDE_D static float2* odd_stages() {
    __shared__ float2 buf[7 * (N % 2 ? 1 : 0) * kFfStageThreads + 1];
    return buf + threadIdx.x;
  }
  GBDE_D static FfVec<N> ld(int j) {
    FfVec<N> v;
    const ulonglong2* sp = pair_stages();
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const ulonglong2 x = sp[(j * Q + q) * kFfStageThreads];
      v.h[q].v = x.x;
      v.l[q].v = x.y;
    }
    if constexpr (N % 2) {
      const float2 x = odd_stages()[j * kFfStageThreads];
      v.o = ff(x.x, x.y);
    }
    return v;
  }
  GBDE_D static void st(int j, const ff* x) {
    ulonglong2* sp = pair_stages();
#pragma unroll
    for (int q = 0; q < Q; ++q)
      sp[(j * Q + q) * kFfStageThreads] =
          make_ulonglong2(f2_pack(x[2 * q].hi, x[2 * q + 1].hi).v,
                          f2_pack(x[2 * q].lo, x[2 * q + 1].lo).v);
    if constexpr (N % 2) odd_stages()[j * kFfStageThreads] = make_float2(x[N - 1].hi, x[N - 1].lo);
  }

  GBDE_D void init(const ff* u0, const ff* p, int& nf) {
#pragma unroll
    for (int k = 0; k < M::NP; ++k) pd[k] = (double)p[k];
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = u0[c];
    M::f(F0, uu, p);
    ++nf;
    fresh = true;
  }

  // One attempted step.  f(uu) and the Jacobian are evaluated afresh on every
  // attempt instead of being kept across a rejection: keeping them would hold
  // 3N + 2N^2 registers through the stage loop for the ~15% of attempts that
  // follow a rejection.  nf counts f(uu) once per accepted state, as a caching
  // implementation would evaluate it.
  GBDE_D double attempt(double dt, const ff* p, double abstol, double reltol, int& nf) {
    if (!fresh) {
      ++nf;
      fresh = true;
    }
    // W = I/(h gamma) - J(uu) and its LU in FP64
    SmallLU<N> W;
    {
      double ud[N], J[N][N];
#pragma unroll
      for (int c = 0; c < N; ++c) ud[c] = f2d_bits(uu[c].hi) + f2d_bits(uu[c].lo);
      M::jac(J, ud, pd);
      const double dg0 = rcp64(dt) * (1.0 / K::g);
#pragma unroll
      for (int r = 0; r < N; ++r)
#pragma unroll
        for (int c = 0; c < N; ++c) W.A[r][c] = r == c ? dg0 - J[r][c] : -J[r][c];
    }
    W.factor();
    FfLU<N> L;
    L.from(W);
    const ff iht = ff_split(rcp64(dt));
    const RodasFfTab& tb = c_rodas_ff[RodasFfIdx<Tag>::v];
    FfVec<N> uv;
    uv.from(uu);
    ff y[N], s[N];
#pragma unroll 1
    for (int i = 0; i < 8; ++i) {
      // stage argument: u0 for stage 1, a fresh combination for stages 2-6; for
      // 7 and 8 the previous argument plus the previous stage (a_7j = a_6j,
      // a_76 = 1, a_8j = a_7j, a_87 = 1)
      FfVecAcc<N> ya, ca;
      const bool fresh_arg = i <= 5;
      if (fresh_arg) {
        ya.set(uv);
      } else {
        FfVec<N> yv;
        yv.from(y);
        ya.set(yv);
      }
      ca.zero();
#pragma unroll 1
      for (int j = 0; j < i; ++j) {
        const ff cij = tb.rc[i][j];
        const ff aij = tb.ra[fresh_arg ? i : 0][fresh_arg ? j : 0];
        const FfVec<N> sj = ld(j);
        if (fresh_arg) ya.fma(aij, sj);
        else if (j == i - 1) ya.add(sj);
        ca.fma(cij, sj);
      }
      ff fy[N], r[N];
      ya.get(y);
      M::f(fy, y, p);
      if (i > 0) {
        ff cs[N];
        ca.get(cs);
        FfVec<N> fv, cv;
        fv.from(fy);
        cv.from(cs);
        FfVecAcc<N> ra;
        ra.set(fv);
        ra.fma(iht, cv);
        ra.get(r);
      } else {
#pragma unroll
        for (int c = 0; c < N; ++c) r[c] = fy[c];
      }
      L.solve(r);
      if (i < 7) {
        st(i, r);
      } else {
#pragma unroll
        for (int c = 0; c < N; ++c) s[c] = r[c];
      }
    }
    nf += 7;
    // y1 = U_7 + u_8; error estimate u_8.  The norm's ratios
    // u_8 / (abstol + reltol max(|u0|, |y1|)) are FP32 on the leading parts
    // (as Tsit5FF); their squares accumulate in FP64.
    const float atf = tol_f32(abstol), rtf = tol_f32(reltol);
    double ms = 0.0;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      FfAcc a;
      a.set(y[c]);
      a.add(s[c]);
      un[c] = a.get();
      const float m = fmaxf(fabsf(uu[c].hi), fabsf(un[c].hi));
      const double e = f2d_bits(norm_ratio(s[c].hi, fmaf(rtf, m, atf)));
      ms = fma(e, e, ms);
    }
    return ms * (1.0 / N);
  }

  // y(theta) = y0 + theta (y1 - y0) + sum_j e_j u_j with
  // e_j = theta (1 - theta) (H2_j + theta H3_j + theta^2 H4_j) (as RodasAlg::interp),
  // all in pair arithmetic; the loop over j reads the coefficients from the
  // constant table.
  GBDE_D void interp(double th, double, ff* out, const ff*, int&) {
    const RodasFfTab& tb = c_rodas_ff[RodasFfIdx<Tag>::v];
    const ff tt = ff_split(th);
    const ff w = tt * (ff(1.0f, 0.0f) - tt);
    ff du[N];
#pragma unroll
    for (int c = 0; c < N; ++c) du[c] = un[c] - uu[c];
    FfVec<N> uv, dv;
    uv.from(uu);
    dv.from(du);
    FfVecAcc<N> a;
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

  GBDE_D void accept(const ff*, int&) {
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = un[c];
    fresh = false;
  }
};

}  // namespace gbde
