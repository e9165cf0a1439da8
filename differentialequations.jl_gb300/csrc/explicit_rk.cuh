// explicit_rk.cuh -- Tsit5 and Vern7 single-trajectory steppers.
//
// These replace OrdinaryDiffEq's perform_step! for Tsit5 (qa.jl:119; used at
// test/core.jl:14,32) and Vern7 (qa.jl:126).  Coefficients: tableaus.h.
// State and stages live in registers (one trajectory per thread).
#pragma once
#include "solver.cuh"
#include "tableaus.h"

namespace gbde {

// EIG: also estimate the spectral radius of the Jacobian along the step for
// run-time stiffness detection (AutoSwitchAlg, autoswitch.cuh): Hairer &
// Wanner II (IV.2) with the infinity norm, from the last two stages and their
// arguments, eig = max_c |(k7_c - k6_c) / (y1_c - g6_c)| (NaN if any ratio is
// NaN, as a maximum over a vector with a NaN).
template <class M, class T, bool EIG = false>
struct Tsit5Alg {
  static constexpr int ORDER = 5, ALG_ID = GBDE_ALG_TSIT5, N = M::N;
  double eig;  // written by attempt() when EIG
  // FP32 path: the state is the unevaluated sum uu + lo (compensated), so
  // the per-step rounding of u + h*sum(b k) does not accumulate.
  static constexpr bool CMP = sizeof(T) == 4;
  T uu[N], un[N], k1[N], k2[N], k3[N], k4[N], k5[N], k6[N], k7[N];
  T lo[N], lon[N];

  GBDE_D T at(int c, T inc) const {
    if constexpr (CMP) return uu[c] + (lo[c] + inc);
    else return uu[c] + inc;
  }
  GBDE_D void advance(int c, T inc) {
    if constexpr (CMP) two_sum_t(uu[c], lo[c] + inc, un[c], lon[c]);
    else un[c] = uu[c] + inc;
  }

  GBDE_D const T* u() const { return uu; }
  GBDE_D const T* unew() const { return un; }
  GBDE_D const T* f0() const { return k1; }

  GBDE_D void init(const T* u0, const T* p, int& nf) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = u0[c];
      lo[c] = T(0);
    }
    M::f(k1, uu, p);
    ++nf;
  }

  GBDE_D double attempt(double dt, const T* p, double abstol, double reltol, int& nf) {
    using namespace tab::tsit5;
    const T h = (T)dt;
    T y[N];
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = at(c, h * (T(a21) * k1[c]));
    M::f(k2, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = at(c, h * (T(a31) * k1[c] + T(a32) * k2[c]));
    M::f(k3, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a41) * k1[c] + T(a42) * k2[c] + T(a43) * k3[c]));
    M::f(k4, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a51) * k1[c] + T(a52) * k2[c] + T(a53) * k3[c] + T(a54) * k4[c]));
    M::f(k5, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a61) * k1[c] + T(a62) * k2[c] + T(a63) * k3[c] + T(a64) * k4[c] +
                          T(a65) * k5[c]));
    M::f(k6, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      advance(c, h * (T(a71) * k1[c] + T(a72) * k2[c] + T(a73) * k3[c] + T(a74) * k4[c] +
                      T(a75) * k5[c] + T(a76) * k6[c]));
    M::f(k7, un, p);
    nf += 6;
    if constexpr (EIG) {  // y holds the 6th stage's argument
      double mx = 0.0;
      bool nan = false;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const double r =
            fabs(((double)k7[c] - (double)k6[c]) / ((double)un[c] - (double)y[c]));
        nan |= r != r;
        mx = fmax(mx, r);
      }
      eig = nan ? __longlong_as_double(0x7ff8000000000000ll) : mx;
    }
    T err[N];
#pragma unroll
    for (int c = 0; c < N; ++c)
      err[c] = h * (T(bt1) * k1[c] + T(bt2) * k2[c] + T(bt3) * k3[c] + T(bt4) * k4[c] +
                    T(bt5) * k5[c] + T(bt6) * k6[c] + T(bt7) * k7[c]);
    return err_ms<N>(err, uu, un, abstol, reltol);
  }

  // continue at u0 with f(u0) = f0 already known (a switch of methods)
  GBDE_D void init_from(const T* u0, const T* f0, const T*) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = u0[c];
      lo[c] = T(0);
      k1[c] = f0[c];
    }
  }

  GBDE_D void interp(double th, double dt, T* out, const T*, int&) {
    using namespace tab::tsit5;
    const double t2 = th * th;
    const T b1 = (T)(r11 * th * (th - r12) * (t2 - r13 * th + r14));
    const T b2 = (T)(r21 * t2 * (t2 - r22 * th + r23));
    const T b3 = (T)(r31 * t2 * (t2 - r32 * th + r33));
    const T b4 = (T)(r41 * (th - r42) * (th - r43) * t2);
    const T b5 = (T)(r51 * (th - r52) * (th - r53) * t2);
    const T b6 = (T)(r61 * (th - r62) * (th - r63) * t2);
    const T b7 = (T)(r71 * (th - r72) * (th - r73) * t2);
    const T h = (T)dt;
#pragma unroll
    for (int c = 0; c < N; ++c)
      out[c] = at(c, h * (b1 * k1[c] + b2 * k2[c] + b3 * k3[c] + b4 * k4[c] + b5 * k5[c] +
                          b6 * k6[c] + b7 * k7[c]));
  }

  GBDE_D void accept(const T*, int&) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = un[c];
      if constexpr (CMP) lo[c] = lon[c];
      k1[c] = k7[c];
    }
  }
};

template <class M, class T>
struct Vern7Alg {
  static constexpr int ORDER = 7, ALG_ID = GBDE_ALG_VERN7, N = M::N;
  static constexpr bool CMP = sizeof(T) == 4;  // compensated FP32 state (as Tsit5Alg)
  T uu[N], un[N], k1[N], k4[N], k5[N], k6[N], k7[N], k8[N], k9[N], k10[N], k11[N];
  T k2[N], k3[N];
  T lo[N], lon[N];
  bool have11;

  GBDE_D T at(int c, T inc) const {
    if constexpr (CMP) return uu[c] + (lo[c] + inc);
    else return uu[c] + inc;
  }
  GBDE_D void advance(int c, T inc) {
    if constexpr (CMP) two_sum_t(uu[c], lo[c] + inc, un[c], lon[c]);
    else un[c] = uu[c] + inc;
  }

  GBDE_D const T* u() const { return uu; }
  GBDE_D const T* unew() const { return un; }
  GBDE_D const T* f0() const { return k1; }

  GBDE_D void init(const T* u0, const T* p, int& nf) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = u0[c];
      lo[c] = T(0);
    }
    M::f(k1, uu, p);
    ++nf;
    have11 = false;
  }

  GBDE_D double attempt(double dt, const T* p, double abstol, double reltol, int& nf) {
    using namespace tab::vern7;
    const T h = (T)dt;
    T y[N];
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = at(c, h * (T(a21) * k1[c]));
    M::f(k2, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = at(c, h * (T(a31) * k1[c] + T(a32) * k2[c]));
    M::f(k3, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = at(c, h * (T(a41) * k1[c] + T(a43) * k3[c]));
    M::f(k4, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a51) * k1[c] + T(a53) * k3[c] + T(a54) * k4[c]));
    M::f(k5, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a61) * k1[c] + T(a63) * k3[c] + T(a64) * k4[c] + T(a65) * k5[c]));
    M::f(k6, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a71) * k1[c] + T(a73) * k3[c] + T(a74) * k4[c] + T(a75) * k5[c] +
                          T(a76) * k6[c]));
    M::f(k7, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a81) * k1[c] + T(a83) * k3[c] + T(a84) * k4[c] + T(a85) * k5[c] +
                          T(a86) * k6[c] + T(a87) * k7[c]));
    M::f(k8, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a91) * k1[c] + T(a93) * k3[c] + T(a94) * k4[c] + T(a95) * k5[c] +
                          T(a96) * k6[c] + T(a97) * k7[c] + T(a98) * k8[c]));
    M::f(k9, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c)
      y[c] = at(c, h * (T(a101) * k1[c] + T(a103) * k3[c] + T(a104) * k4[c] +
                          T(a105) * k5[c] + T(a106) * k6[c] + T(a107) * k7[c]));
    M::f(k10, y, p);
    nf += 9;
    T err[N];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      advance(c, h * (T(b1) * k1[c] + T(b4) * k4[c] + T(b5) * k5[c] + T(b6) * k6[c] +
                      T(b7) * k7[c] + T(b8) * k8[c] + T(b9) * k9[c]));
      err[c] = h * (T(b1 - bh1) * k1[c] + T(b4 - bh4) * k4[c] + T(b5 - bh5) * k5[c] +
                    T(b6 - bh6) * k6[c] + T(b7 - bh7) * k7[c] + T(b8) * k8[c] + T(b9) * k9[c] -
                    T(bh10) * k10[c]);
    }
    have11 = false;
    return err_ms<N>(err, uu, un, abstol, reltol);
  }

  // 7th-order dense output u(theta) = y0 + h sum_j D_j(theta) K_j
  // (dense_coeffs.h, vern7l) over K1, K4..K9, K11 = f(t+h, y1) and four lazy
  // stages: K12..K14 on the 5th-order extension at theta = 0.12, 0.25, 0.78,
  // then K15..K18 on the degree-6 interpolant through them at theta = 0.11,
  // 0.22, 0.55, 0.75.  The lazy stages are evaluated for each save point and
  // each of K15..K18 is folded into the sum as soon as it exists, so that few
  // stage vectors are live at once (the kernel's register count is set by its
  // peak).
  GBDE_D void interp(double th, double dt, T* out, const T* p, int& nf) {
    using namespace tab::vern7l;
    if (!have11) {
      M::f(k11, un, p);
      ++nf;
      have11 = true;
    }
    const T h = (T)dt;
#define GBDE_V7D(j)                                                                          \
  (T)(th * (D##j##_1 + th * (D##j##_2 + th * (D##j##_3 + th * (D##j##_4 +                    \
      th * (D##j##_5 + th * (D##j##_6 + th * D##j##_7)))))))
    T acc[N];
    {
      const T w1 = GBDE_V7D(1), w4 = GBDE_V7D(4), w5 = GBDE_V7D(5), w6 = GBDE_V7D(6);
      const T w7 = GBDE_V7D(7), w8 = GBDE_V7D(8), w9 = GBDE_V7D(9), w11 = GBDE_V7D(11);
#pragma unroll
      for (int c = 0; c < N; ++c)
        acc[c] = w1 * k1[c] + w4 * k4[c] + w5 * k5[c] + w6 * k6[c] + w7 * k7[c] + w8 * k8[c] +
                 w9 * k9[c] + w11 * k11[c];
    }
    T k12[N], k13[N], k14[N], y[N], k[N];
#define GBDE_V7L1(i, c)                                                                         \
  (T(L1_##i##_1) * k1[c] + T(L1_##i##_4) * k4[c] + T(L1_##i##_5) * k5[c] +                      \
   T(L1_##i##_6) * k6[c] + T(L1_##i##_7) * k7[c] + T(L1_##i##_8) * k8[c] +                      \
   T(L1_##i##_9) * k9[c] + T(L1_##i##_10) * k10[c] + T(L1_##i##_11) * k11[c])
#define GBDE_V7L2(i, c)                                                                         \
  (T(L2_##i##_1) * k1[c] + T(L2_##i##_4) * k4[c] + T(L2_##i##_5) * k5[c] +                      \
   T(L2_##i##_6) * k6[c] + T(L2_##i##_7) * k7[c] + T(L2_##i##_8) * k8[c] +                      \
   T(L2_##i##_9) * k9[c] + T(L2_##i##_11) * k11[c] + T(L2_##i##_12) * k12[c] +                  \
   T(L2_##i##_13) * k13[c] + T(L2_##i##_14) * k14[c])
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = at(c, h * GBDE_V7L1(1, c));
    M::f(k12, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = at(c, h * GBDE_V7L1(2, c));
    M::f(k13, y, p);
#pragma unroll
    for (int c = 0; c < N; ++c) y[c] = at(c, h * GBDE_V7L1(3, c));
    M::f(k14, y, p);
#define GBDE_V7LAZY2(i, j)                                                                      \
  _Pragma("unroll") for (int c = 0; c < N; ++c) y[c] = at(c, h * GBDE_V7L2(i, c));              \
  M::f(k, y, p);                                                                                \
  {                                                                                             \
    const T w = GBDE_V7D(j);                                                                    \
    _Pragma("unroll") for (int c = 0; c < N; ++c) acc[c] += w * k[c];                           \
  }
    GBDE_V7LAZY2(1, 15)
    GBDE_V7LAZY2(2, 16)
    GBDE_V7LAZY2(3, 17)
    GBDE_V7LAZY2(4, 18)
#undef GBDE_V7LAZY2
#undef GBDE_V7L1
#undef GBDE_V7L2
#undef GBDE_V7D
    nf += 7;
#pragma unroll
    for (int c = 0; c < N; ++c) out[c] = at(c, h * acc[c]);
  }

  GBDE_D void accept(const T* p, int& nf) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      uu[c] = un[c];
      if constexpr (CMP) lo[c] = lon[c];
    }
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

}  // namespace gbde
