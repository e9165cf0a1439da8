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
#include "ff.cuh"
#include "rosenbrock.cuh"

namespace gbde {

// Split a double into a pair without FP64 arithmetic: hi keeps the leading 24
// significant bits (truncated), lo the remaining 29 bits rounded to 24 (one
// integer-to-float conversion and an exact power-of-two scaling).  |lo| < ulp(hi).
// |d| below 2^-126 gives a signed zero (below 2^-74 lo is dropped); |d| >= 2^128
// gives an infinity (NaN stays NaN).
GBDE_D ff ff_split(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const unsigned sign = hw & 0x80000000u;
  const int ex = (int)((hw >> 20) & 0x7ffu);
  if (ex < 897) return ff(__uint_as_float(sign), 0.0f);
  if (ex > 1150) {
    const bool nan = ex == 2047 && (b << 12) != 0ull;
    return ff(__uint_as_float(nan ? 0x7fc00000u : (sign | 0x7f800000u)), 0.0f);
  }
  const unsigned m23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
  const float hi = __uint_as_float(sign | ((unsigned)(ex - 896) << 23) | m23);
  float lo = 0.0f;
  if (ex >= 949) lo = xmul(__uint2float_rn(lw & 0x1fffffffu), __uint_as_float((unsigned)(ex - 948) << 23));
  return ff(hi, sign ? -lo : lo);
}

// Unnormalised accumulator of a sum of pair products: value = s + e.  Each term
// costs one TwoProd with cross terms and one TwoSum; get() renormalises once.
struct FfAcc {
  float s, e;
  GBDE_D void set(ff x) {
    s = x.hi;
    e = x.lo;
  }
  GBDE_D void fma(ff a, ff b) {  // += a b
    const float p = xmul(a.hi, b.hi);
    float pe = xfma(a.hi, b.hi, -p);
    pe = xfma(a.hi, b.lo, xfma(a.lo, b.hi, pe));
    const float t = xadd(s, p);
    const float bb = xadd(t, -s);
    const float err = xadd(xadd(s, -xadd(t, -bb)), xadd(p, -bb));
    s = t;
    e = xadd(e, xadd(err, pe));
  }
  GBDE_D void add(ff x) {  // += x
    const float t = xadd(s, x.hi);
    const float bb = xadd(t, -s);
    const float err = xadd(xadd(s, -xadd(t, -bb)), xadd(x.hi, -bb));
    s = t;
    e = xadd(e, xadd(err, x.lo));
  }
  GBDE_D ff get() const {  // TwoSum renormalisation (|e| may exceed |s| after cancellation)
    const float t = xadd(s, e);
    const float bb = xadd(t, -s);
    const float err = xadd(xadd(s, -xadd(t, -bb)), xadd(e, -bb));
    return ff(t, err);
  }
};

// ---- two state components per instruction
// Blackwell's paired FP32 arithmetic (add / sub / mul / fma .rn.f32x2) takes
// two FP32 values in one 64-bit register and rounds each exactly as the scalar
// instruction would, so pairing state components (0,1), (2,3), ... halves the
// issue slots of the pair sums while giving bit-identical results.  The
// product is carried negated (pn = -p) because there is no paired negation.
struct F2 {
  unsigned long long v;
};
GBDE_D F2 f2_pack(float lo, float hi) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
GBDE_D void f2_unpack(F2 a, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
GBDE_D F2 f2_add(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
GBDE_D F2 f2_sub(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
GBDE_D F2 f2_mul(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
GBDE_D F2 f2_fma(F2 a, F2 b, F2 c) {  // a b + c
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}

// FfAcc for two components at once: (s, e) hold components c and c + 1.
struct FfAcc2 {
  F2 s, e;
  GBDE_D void set(F2 h, F2 l) {
    s = h;
    e = l;
  }
  // += a (one pair coefficient for both) * b (hi parts bh, lo parts bl);
  // ah = (a.hi, a.hi), al = (a.lo, a.lo), ahn = (-a.hi, -a.hi)
  GBDE_D void fma(F2 ah, F2 al, F2 ahn, F2 bh, F2 bl) {
    const F2 pn = f2_mul(ahn, bh);                       // -p
    F2 pe = f2_fma(ah, bh, pn);                          // a.hi b.hi - p, exactly
    pe = f2_fma(ah, bl, f2_fma(al, bh, pe));
    const F2 t = f2_sub(s, pn);                          // s + p
    const F2 bb = f2_sub(t, s);
    const F2 err = f2_sub(f2_sub(s, f2_sub(t, bb)), f2_add(pn, bb));  // (s-(t-bb)) + (p-bb)
    s = t;
    e = f2_add(e, f2_add(err, pe));
  }
  GBDE_D void add(F2 xh, F2 xl) {  // += x
    const F2 t = f2_add(s, xh);
    const F2 bb = f2_sub(t, s);
    const F2 err = f2_add(f2_sub(s, f2_sub(t, bb)), f2_sub(xh, bb));
    s = t;
    e = f2_add(e, f2_add(err, xl));
  }
  GBDE_D void get(ff& x0, ff& x1) const {  // TwoSum renormalisation, as FfAcc::get
    const F2 t = f2_add(s, e);
    const F2 bb = f2_sub(t, s);
    const F2 err = f2_add(f2_sub(s, f2_sub(t, bb)), f2_sub(e, bb));
    f2_unpack(t, x0.hi, x1.hi);
    f2_unpack(err, x0.lo, x1.lo);
  }
};

// A vector of N pairs as Q = N/2 paired halves (hi of c, c+1; lo of c, c+1)
// plus the odd last component.
template <int N>
struct FfVec {
  static constexpr int Q = N / 2;
  F2 h[Q > 0 ? Q : 1], l[Q > 0 ? Q : 1];
  ff o;
  GBDE_D void from(const ff* x) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      h[q] = f2_pack(x[2 * q].hi, x[2 * q + 1].hi);
      l[q] = f2_pack(x[2 * q].lo, x[2 * q + 1].lo);
    }
    if constexpr (N % 2) o = x[N - 1];
  }
};

// Accumulator over a whole vector: FfAcc2 for the pairs, FfAcc for the odd one.
template <int N>
struct FfVecAcc {
  static constexpr int Q = N / 2;
  FfAcc2 v[Q > 0 ? Q : 1];
  FfAcc w;
  GBDE_D void set(const FfVec<N>& x) {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q].set(x.h[q], x.l[q]);
    if constexpr (N % 2) w.set(x.o);
  }
  GBDE_D void zero() {
    const F2 z = f2_pack(0.0f, 0.0f);
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q].set(z, z);
    if constexpr (N % 2) w.set(ff(0.0f, 0.0f));
  }
  GBDE_D void fma(ff a, const FfVec<N>& b) {
    const F2 ah = f2_pack(a.hi, a.hi), al = f2_pack(a.lo, a.lo), ahn = f2_pack(-a.hi, -a.hi);
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q].fma(ah, al, ahn, b.h[q], b.l[q]);
    if constexpr (N % 2) w.fma(a, b.o);
  }
  GBDE_D void add(const FfVec<N>& b) {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q].add(b.h[q], b.l[q]);
    if constexpr (N % 2) w.add(b.o);
  }
  GBDE_D void get(ff* out) const {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q].get(out[2 * q], out[2 * q + 1]);
    if constexpr (N % 2) out[N - 1] = w.get();
  }
};

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
    // y1 = U_7 + u_8; error estimate u_8, norm in FP64
    double ms = 0.0;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      FfAcc a;
      a.set(y[c]);
      a.add(s[c]);
      un[c] = a.get();
      const float m = fmaxf(fabsf(uu[c].hi), fabsf(un[c].hi));
      const double e = f2d_bits(s[c].hi) * rcp64(abstol + reltol * f2d_bits(m));
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
