// vern7_ff.cuh -- Vern7 in FP32 pairs (the F32X2 precision) for models of up
// to three states.
//
// Same method as Vern7Alg (explicit_rk.cuh; OrdinaryDiffEq's Vern7,
// test/qa/qa.jl:126): Verner's 10-stage 7(6) pair and this library's
// 7th-order dense output with the lazily evaluated f(u1) and seven lazy
// stages.  The work is placed
// as in Tsit5FF (tsit5_ff.cuh): the stage derivatives are kept pre-scaled,
// hk_j = h k_j, in paired FP32 registers; every stage argument, the new state,
// the error estimate and the dense output is one unnormalised accumulation
// (FfVecAcc); h and theta enter through the integer-pipe split; the norm's
// ratios are FP32 on the leading parts with their squares accumulated in FP64.
#pragma once
#include "ff_vec.cuh"
#include "explicit_rk.cuh"

namespace gbde {

template <class M>
struct Vern7FF {
  using T = ff;
  static constexpr int ORDER = 7, ALG_ID = GBDE_ALG_VERN7, N = M::N;
  // the driver computes a step's end before the attempt (small ensembles run
  // one warp per SM sub-partition, where step latency is the time)
  static constexpr bool EARLY_TIME = true;
  ff uu[N], un[N];
  ff k1[N];        // f(uu)
  ff k11[N];       // f(un), evaluated for the dense output only
  FfVec<N> hk[11]; // h k_1 .. h k_11 of the current attempt (hk[10] once have11)
  bool have11;

  GBDE_D const ff* u() const { return uu; }
  GBDE_D const ff* unew() const { return un; }
  GBDE_D const ff* f0() const { return k1; }

  GBDE_D void init(const ff* u0, const ff* p, int& nf) {
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = u0[c];
    M::f(k1, uu, p);
    ++nf;
    have11 = false;
  }

  GBDE_D double attempt(double dt, const ff* p, double abstol, double reltol, int& nf) {
    using namespace tab::vern7;
    constexpr ff A21 = ff(a21), A31 = ff(a31), A32 = ff(a32), A41 = ff(a41), A43 = ff(a43);
    constexpr ff A51 = ff(a51), A53 = ff(a53), A54 = ff(a54);
    constexpr ff A61 = ff(a61), A63 = ff(a63), A64 = ff(a64), A65 = ff(a65);
    constexpr ff A71 = ff(a71), A73 = ff(a73), A74 = ff(a74), A75 = ff(a75), A76 = ff(a76);
    constexpr ff A81 = ff(a81), A83 = ff(a83), A84 = ff(a84), A85 = ff(a85), A86 = ff(a86),
                 A87 = ff(a87);
    constexpr ff A91 = ff(a91), A93 = ff(a93), A94 = ff(a94), A95 = ff(a95), A96 = ff(a96),
                 A97 = ff(a97), A98 = ff(a98);
    constexpr ff A101 = ff(a101), A103 = ff(a103), A104 = ff(a104), A105 = ff(a105),
                 A106 = ff(a106), A107 = ff(a107);
    constexpr ff B1 = ff(b1), B4 = ff(b4), B5 = ff(b5), B6 = ff(b6), B7 = ff(b7), B8 = ff(b8),
                 B9 = ff(b9);
    constexpr ff E1 = ff(b1 - bh1), E4 = ff(b4 - bh4), E5 = ff(b5 - bh5), E6 = ff(b6 - bh6),
                 E7 = ff(b7 - bh7), E8 = ff(b8), E9 = ff(b9), E10 = ff(-bh10);
    const ff h = ff_split(dt);
    FfVec<N> uv;
    uv.from(uu);
    ff y[N], k[N];
    FfVecAcc<N> a;
    hk[0] = ff_scale<N>(h, k1);
#define GBDE_V7FF_STAGE(dst)  \
  a.get(y);                   \
  M::f(k, y, p);              \
  hk[dst] = ff_scale<N>(h, k);
    a.set(uv);
    a.fma(A21, hk[0]);
    GBDE_V7FF_STAGE(1)
    a.set(uv);
    a.fma(A31, hk[0]);
    a.fma(A32, hk[1]);
    GBDE_V7FF_STAGE(2)
    a.set(uv);
    a.fma(A41, hk[0]);
    a.fma(A43, hk[2]);
    GBDE_V7FF_STAGE(3)
    a.set(uv);
    a.fma(A51, hk[0]);
    a.fma(A53, hk[2]);
    a.fma(A54, hk[3]);
    GBDE_V7FF_STAGE(4)
    a.set(uv);
    a.fma(A61, hk[0]);
    a.fma(A63, hk[2]);
    a.fma(A64, hk[3]);
    a.fma(A65, hk[4]);
    GBDE_V7FF_STAGE(5)
    a.set(uv);
    a.fma(A71, hk[0]);
    a.fma(A73, hk[2]);
    a.fma(A74, hk[3]);
    a.fma(A75, hk[4]);
    a.fma(A76, hk[5]);
    GBDE_V7FF_STAGE(6)
    a.set(uv);
    a.fma(A81, hk[0]);
    a.fma(A83, hk[2]);
    a.fma(A84, hk[3]);
    a.fma(A85, hk[4]);
    a.fma(A86, hk[5]);
    a.fma(A87, hk[6]);
    GBDE_V7FF_STAGE(7)
    a.set(uv);
    a.fma(A91, hk[0]);
    a.fma(A93, hk[2]);
    a.fma(A94, hk[3]);
    a.fma(A95, hk[4]);
    a.fma(A96, hk[5]);
    a.fma(A97, hk[6]);
    a.fma(A98, hk[7]);
    GBDE_V7FF_STAGE(8)
    a.set(uv);
    a.fma(A101, hk[0]);
    a.fma(A103, hk[2]);
    a.fma(A104, hk[3]);
    a.fma(A105, hk[4]);
    a.fma(A106, hk[5]);
    a.fma(A107, hk[6]);
    GBDE_V7FF_STAGE(9)
#undef GBDE_V7FF_STAGE
    nf += 9;
    // u1 = u0 + sum_j b_j h k_j
    a.set(uv);
    a.fma(B1, hk[0]);
    a.fma(B4, hk[3]);
    a.fma(B5, hk[4]);
    a.fma(B6, hk[5]);
    a.fma(B7, hk[6]);
    a.fma(B8, hk[7]);
    a.fma(B9, hk[8]);
    a.get(un);
    // error estimate sum_j (b_j - bhat_j) h k_j, norm ratios in FP32, squares in FP64
    ff err[N];
    a.zero();
    a.fma(E1, hk[0]);
    a.fma(E4, hk[3]);
    a.fma(E5, hk[4]);
    a.fma(E6, hk[5]);
    a.fma(E7, hk[6]);
    a.fma(E8, hk[7]);
    a.fma(E9, hk[8]);
    a.fma(E10, hk[9]);
    a.get(err);
    have11 = false;
    const float atf = tol_f32(abstol), rtf = tol_f32(reltol);
    double ms = 0.0;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const float m = fmaxf(fabsf(uu[c].hi), fabsf(un[c].hi));
      const double e = f2d_bits(norm_ratio(err[c].hi, fmaf(rtf, m, atf)));
      ms = fma(e, e, ms);
    }
    return ms * (1.0 / N);
  }

  // The interpolant's seven lazy stages (as Vern7Alg::lazy_stages), in pair
  // arithmetic: K12..K14 on the 5th-order extension, K15..K18 on the degree-6
  // interpolant through them (per save point, as in Vern7Alg).
  GBDE_D void lazy_stages(double dt, const ff* p, int& nf, FfVec<N>* hl) {
    using namespace tab::vern7l;
    const ff h = ff_split(dt);
    FfVec<N> uv, l1[3];
    uv.from(uu);
    FfVecAcc<N> a;
    ff y[N], k[N];
#define GBDE_V7FF_L1(i)                                                                          \
  a.set(uv);                                                                                     \
  a.fma(ff(L1_##i##_1), hk[0]);                                                                  \
  a.fma(ff(L1_##i##_4), hk[3]);                                                                  \
  a.fma(ff(L1_##i##_5), hk[4]);                                                                  \
  a.fma(ff(L1_##i##_6), hk[5]);                                                                  \
  a.fma(ff(L1_##i##_7), hk[6]);                                                                  \
  a.fma(ff(L1_##i##_8), hk[7]);                                                                  \
  a.fma(ff(L1_##i##_9), hk[8]);                                                                  \
  a.fma(ff(L1_##i##_10), hk[9]);                                                                 \
  a.fma(ff(L1_##i##_11), hk[10]);                                                                \
  a.get(y);                                                                                      \
  M::f(k, y, p);                                                                                 \
  l1[i - 1] = ff_scale<N>(h, k);
    GBDE_V7FF_L1(1)
    GBDE_V7FF_L1(2)
    GBDE_V7FF_L1(3)
#undef GBDE_V7FF_L1
#define GBDE_V7FF_L2(i)                                                                          \
  a.set(uv);                                                                                     \
  a.fma(ff(L2_##i##_1), hk[0]);                                                                  \
  a.fma(ff(L2_##i##_4), hk[3]);                                                                  \
  a.fma(ff(L2_##i##_5), hk[4]);                                                                  \
  a.fma(ff(L2_##i##_6), hk[5]);                                                                  \
  a.fma(ff(L2_##i##_7), hk[6]);                                                                  \
  a.fma(ff(L2_##i##_8), hk[7]);                                                                  \
  a.fma(ff(L2_##i##_9), hk[8]);                                                                  \
  a.fma(ff(L2_##i##_11), hk[10]);                                                                \
  a.fma(ff(L2_##i##_12), l1[0]);                                                                 \
  a.fma(ff(L2_##i##_13), l1[1]);                                                                 \
  a.fma(ff(L2_##i##_14), l1[2]);                                                                 \
  a.get(y);                                                                                      \
  M::f(k, y, p);                                                                                 \
  hl[i - 1] = ff_scale<N>(h, k);
    GBDE_V7FF_L2(1)
    GBDE_V7FF_L2(2)
    GBDE_V7FF_L2(3)
    GBDE_V7FF_L2(4)
#undef GBDE_V7FF_L2
    nf += 7;
  }

  // y(theta) = y0 + sum_j w_j(theta) h k_j with w_j(theta) = theta (D_j1 +
  // theta (D_j2 + ... + theta D_j7)) (as Vern7Alg::interp), in pair arithmetic;
  // f(u1) is evaluated on the first call of a step, the lazy stages on each.
  GBDE_D void interp(double th, double dt, ff* out, const ff* p, int& nf) {
    using namespace tab::vern7l;
    if (!have11) {
      M::f(k11, un, p);
      ++nf;
      hk[10] = ff_scale<N>(ff_split(dt), k11);
      have11 = true;
    }
    FfVec<N> hl[4];
    lazy_stages(dt, p, nf, hl);
    const ff t = ff_split(th);
#define GBDE_V7FF_W(j)                                                                           \
  (t * (ff(D##j##_1) +                                                                           \
        t * (ff(D##j##_2) +                                                                      \
             t * (ff(D##j##_3) +                                                                 \
                  t * (ff(D##j##_4) +                                                            \
                       t * (ff(D##j##_5) + t * (ff(D##j##_6) + t * ff(D##j##_7))))))))
    FfVec<N> uv;
    uv.from(uu);
    FfVecAcc<N> a;
    a.set(uv);
    a.fma(GBDE_V7FF_W(1), hk[0]);
    a.fma(GBDE_V7FF_W(4), hk[3]);
    a.fma(GBDE_V7FF_W(5), hk[4]);
    a.fma(GBDE_V7FF_W(6), hk[5]);
    a.fma(GBDE_V7FF_W(7), hk[6]);
    a.fma(GBDE_V7FF_W(8), hk[7]);
    a.fma(GBDE_V7FF_W(9), hk[8]);
    a.fma(GBDE_V7FF_W(11), hk[10]);
    a.fma(GBDE_V7FF_W(15), hl[0]);
    a.fma(GBDE_V7FF_W(16), hl[1]);
    a.fma(GBDE_V7FF_W(17), hl[2]);
    a.fma(GBDE_V7FF_W(18), hl[3]);
#undef GBDE_V7FF_W
    a.get(out);
  }

  GBDE_D void accept(const ff* p, int& nf) {
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = un[c];
    if (have11) {
#pragma unroll
      for (int c = 0; c < N; ++c) k1[c] = k11[c];
    } else {
      M::f(k1, uu, p);
      ++nf;
    }
    have11 = false;
  }
};

// The Vern7 stepper for precision T: the pair stepper above for F32X2 models
// of up to three states, Vern7Alg otherwise.
template <class M, class T, bool PAIR = is_ff<T>::value && (M::N <= 3)>
struct Vern7Sel {
  using type = Vern7Alg<M, T>;
};
template <class M, class T>
struct Vern7Sel<M, T, true> {
  using type = Vern7FF<M>;
};
template <class M, class T>
using Vern7A = typename Vern7Sel<M, T>::type;

}  // namespace gbde
