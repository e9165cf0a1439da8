// tsit5_ff.cuh -- Tsit5 in FP32 pairs (the F32X2 precision) for models of up
// to four states.
//
// Same method as Tsit5Alg (explicit_rk.cuh; OrdinaryDiffEq's Tsit5,
// test/qa/qa.jl:119, used at test/core.jl:14,32): the 7-stage FSAL 5(4) pair
// with its continuous extension.  What differs is where each operation runs:
//
//  * the stage derivatives are kept pre-scaled, hk_j = h k_j, in paired FP32
//    registers (FfVec): every stage argument, the new state, the error
//    estimate and the dense output are one unnormalised accumulation each
//    (FfVecAcc: one TwoProd and one TwoSum per term, two state components per
//    paired instruction, one renormalisation per sum);
//  * h and the dense-output abscissa enter the pair arithmetic through the
//    integer-pipe split (ff_split) instead of FP64 conversions, and the
//    dense-output weights are pair polynomials;
//  * the error norm's ratios err_c / (abstol + reltol max(|u_c|, |u1_c|)) are
//    FP32 on the leading parts; their squares accumulate in FP64.
// GB300 issues one FP64 warp instruction per ~64 cycles on each SM
// sub-partition.  In a small ensemble (one warp per sub-partition) every FP64
// instruction of a step is therefore step latency; here only the norm's
// accumulation and the driver's time and step-size products stay on that
// pipe.
#pragma once
#include "ff_vec.cuh"
#include "explicit_rk.cuh"

namespace gbde {

template <class M>
struct Tsit5FF {
  using T = ff;
  static constexpr int ORDER = 5, ALG_ID = GBDE_ALG_TSIT5, N = M::N;
  // the driver computes a step's end before the attempt (small ensembles run
  // one warp per SM sub-partition, where step latency is the time)
  static constexpr bool EARLY_TIME = true;
  ff uu[N], un[N];
  ff k1[N], k7[N];  // f at the step's start and at its end (first-same-as-last)
  FfVec<N> hk[7];   // h k_j of the current attempt

  GBDE_D const ff* u() const { return uu; }
  GBDE_D const ff* unew() const { return un; }
  GBDE_D const ff* f0() const { return k1; }

  GBDE_D void init(const ff* u0, const ff* p, int& nf) {
#pragma unroll
    for (int c = 0; c < N; ++c) uu[c] = u0[c];
    M::f(k1, uu, p);
    ++nf;
  }

  GBDE_D double attempt(double dt, const ff* p, double abstol, double reltol, int& nf) {
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
    FfVec<N> uv;
    uv.from(uu);
    ff y[N], k[N];
    FfVecAcc<N> a;
    hk[0] = ff_scale<N>(h, k1);
    a.set(uv);
    a.fma(A21, hk[0]);
    a.get(y);
    M::f(k, y, p);
    hk[1] = ff_scale<N>(h, k);
    a.set(uv);
    a.fma(A31, hk[0]);
    a.fma(A32, hk[1]);
    a.get(y);
    M::f(k, y, p);
    hk[2] = ff_scale<N>(h, k);
    a.set(uv);
    a.fma(A41, hk[0]);
    a.fma(A42, hk[1]);
    a.fma(A43, hk[2]);
    a.get(y);
    M::f(k, y, p);
    hk[3] = ff_scale<N>(h, k);
    a.set(uv);
    a.fma(A51, hk[0]);
    a.fma(A52, hk[1]);
    a.fma(A53, hk[2]);
    a.fma(A54, hk[3]);
    a.get(y);
    M::f(k, y, p);
    hk[4] = ff_scale<N>(h, k);
    a.set(uv);
    a.fma(A61, hk[0]);
    a.fma(A62, hk[1]);
    a.fma(A63, hk[2]);
    a.fma(A64, hk[3]);
    a.fma(A65, hk[4]);
    a.get(y);
    M::f(k, y, p);
    hk[5] = ff_scale<N>(h, k);
    a.set(uv);
    a.fma(A71, hk[0]);
    a.fma(A72, hk[1]);
    a.fma(A73, hk[2]);
    a.fma(A74, hk[3]);
    a.fma(A75, hk[4]);
    a.fma(A76, hk[5]);
    a.get(un);
    M::f(k7, un, p);
    hk[6] = ff_scale<N>(h, k7);
    nf += 6;
    // error estimate sum_j btilde_j h k_j (the terms cancel to ~reltol |u|,
    // hence the pair accumulation), norm ratios in FP32, squares in FP64
    ff err[N];
    a.zero();
    a.fma(E1, hk[0]);
    a.fma(E2, hk[1]);
    a.fma(E3, hk[2]);
    a.fma(E4, hk[3]);
    a.fma(E5, hk[4]);
    a.fma(E6, hk[5]);
    a.fma(E7, hk[6]);
    a.get(err);
    const float atf = tol_f32(abstol), rtf = tol_f32(reltol);
    double ms = 0.0;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const float m = fmaxf(fabsf(uu[c].hi), fabsf(un[c].hi));
      const float e = norm_ratio(err[c].hi, fmaf(rtf, m, atf));
      const double ed = f2d_bits(e);
      ms = fma(ed, ed, ms);
    }
    return ms * (1.0 / N);
  }

  // y(theta) = y0 + sum_j b_j(theta) h k_j with Tsit5's interpolation
  // polynomials (as Tsit5Alg::interp), evaluated in pair arithmetic.
  GBDE_D void interp(double th, double, ff* out, const ff*, int&) {
    using namespace tab::tsit5;
    constexpr ff R11 = ff(r11), R12 = ff(r12), R13 = ff(r13), R14 = ff(r14);
    constexpr ff R21 = ff(r21), R22 = ff(r22), R23 = ff(r23);
    constexpr ff R31 = ff(r31), R32 = ff(r32), R33 = ff(r33);
    constexpr ff R41 = ff(r41), R42 = ff(r42), R43 = ff(r43);
    constexpr ff R51 = ff(r51), R52 = ff(r52), R53 = ff(r53);
    constexpr ff R61 = ff(r61), R62 = ff(r62), R63 = ff(r63);
    constexpr ff R71 = ff(r71), R72 = ff(r72), R73 = ff(r73);
    const ff t = ff_split(th), t2 = t * t;
    FfVec<N> uv;
    uv.from(uu);
    FfVecAcc<N> a;
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

  GBDE_D void accept(const ff*, int&) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = un[c];
      k1[c] = k7[c];
    }
  }
};

// The Tsit5 stepper for precision T: the pair stepper above for F32X2 models
// of up to four states, Tsit5Alg otherwise.
template <class M, class T, bool PAIR = is_ff<T>::value && (M::N <= 4)>
struct Tsit5Sel {
  using type = Tsit5Alg<M, T>;
};
template <class M, class T>
struct Tsit5Sel<M, T, true> {
  using type = Tsit5FF<M>;
};
template <class M, class T>
using Tsit5A = typename Tsit5Sel<M, T>::type;

}  // namespace gbde
