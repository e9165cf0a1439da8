// controller.h -- the step-size controller of every adaptive kernel, with
// identical bits on the host and the device.
//
// The PI controller of Hairer-Norsett-Wanner I, Sec. II.4 (Gustafsson's PI
// control), in the form the reference's controller accessors
// (get_proposed_dt / set_proposed_dt!, test/qa/qa.jl:151,187) expose:
//     accept (EEst <= 1):  q = clamp(EEst^beta1 / qold^beta2 / gamma, 1/qmax, 1/qmin)
//                          q = 1 if qsteady_min <= q <= qsteady_max
//                          dt_new = dt / q,  qold = max(EEst, qoldinit)
//     reject:              dt_new = dt / min(1/qmin, EEst^beta1 / gamma)
//     EEst not finite:     dt_new = dt * qmin
// EEst = sqrt(ms), ms the mean square of the scaled error; the accept test
// ms <= 1 stays FP64.  Only the size factor q is evaluated in FP32: it sets
// the size of the next step, not its accuracy, and an FP64 pow() costs about
// as many FP64 instructions as a whole Rosenbrock stage on GB300 (1/61 of the
// FP32 rate).  log2 and exp2 below are this file's own series evaluations,
// built only from correctly rounded IEEE operations (non-contracted multiply /
// add / fma, IEEE division), so the CPU oracle, which includes this header,
// takes exactly the same steps:
//   log2 x = e + 2 atanh(s) / ln 2,  s = (m-1)/(m+1),  x = m 2^e, m in [1/sqrt2, sqrt2)
//   2^y    = 2^k * exp(f ln 2),  k = rint(y), |f| <= 1/2 (Taylor series, degree 7).
// Host code that includes this header must be compiled with -ffp-contract=off.
#pragma once
#ifndef __CUDACC_RTC__
#include <math.h>
#endif
#include "common.cuh"

namespace gbde {

// Controller constants, derived once from the solver options on the host.
struct CtlK {
  float hb1;        // beta1 / 2 (applied to log2 of the mean square)
  float b2;         // beta2
  float inv_gamma;  // 1 / gamma
  float qmax_inv;   // 1 / qmax
  float qmin_inv;   // 1 / qmin
  float qmin;       // qmin (factor after a non-finite error estimate)
  float qs_min, qs_max;
  float lqoldinit;  // log2(qoldinit)
};

// Exact helpers for the series below, on the integer pipe and FP32 adds
// (GB300 runs conversion instructions on its narrow FP64 pipe).
GBDE_HD uint32_t ctl_fbits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  memcpy(&b, &x, sizeof(b));
  return b;
#endif
}
GBDE_HD float ctl_bitsf(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  memcpy(&x, &b, sizeof(x));
  return x;
#endif
}
// 1.5 2^23: adding it to |y| < 2^22 leaves round-to-nearest-even(y) in the
// low bits of the sum's significand
constexpr float kCtlRound = 12582912.0f;
// frexpf for positive normal x: x = m 2^e, m in [0.5, 1)
GBDE_HD float ctl_frexp(float x, int& e) {
  const uint32_t b = ctl_fbits(x);
  e = (int)((b >> 23) & 0xffu) - 126;
  return ctl_bitsf((b & 0x807fffffu) | 0x3f000000u);
}
// (float)i for |i| < 2^22
GBDE_HD float ctl_i2f(int i) { return xadd(ctl_bitsf(0x4b400000u + (uint32_t)i), -kCtlRound); }

GBDE_HD float ctl_log2f(float x) {
  // x > 0 and normal
  int e;
  float m = ctl_frexp(x, e);  // x = m 2^e, m in [0.5, 1): exact
  if (m < 0.707106781f) {
    m = m + m;  // exact
    e -= 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);  // m - 1 exact (Sterbenz); IEEE division
  const float s2 = xmul(s, s);
  // 1 + s2/3 + s2^2/5 + ... + s2^6/13  (s2 <= 0.0295: truncation < 1e-10)
  float pacc = 1.0f / 13.0f;
  pacc = xfma(pacc, s2, 1.0f / 11.0f);
  pacc = xfma(pacc, s2, 1.0f / 9.0f);
  pacc = xfma(pacc, s2, 1.0f / 7.0f);
  pacc = xfma(pacc, s2, 1.0f / 5.0f);
  pacc = xfma(pacc, s2, 1.0f / 3.0f);
  pacc = xfma(pacc, s2, 1.0f);
  const float ln_m = xmul(xadd(s, s), pacc);      // 2 atanh(s) = ln m
  return xfma(ln_m, 1.44269504f, ctl_i2f(e));     // e + ln m / ln 2
}

GBDE_HD float ctl_exp2f(float y) {
  // |y| <= 60 (the callers clamp); k = rint(y) and its integer from one sum
  const float r = xadd(y, kCtlRound);
  const int ki = (int)(ctl_fbits(r) - 0x4b400000u);
  const float k = xadd(r, -kCtlRound);
  const float f = y - k;  // exact, |f| <= 1/2
  const float x = xmul(f, 0.693147182f);  // f ln 2, |x| <= 0.347
  // exp(x) by Taylor series, degree 7 (truncation < 6e-9 relative)
  float pacc = 1.0f / 5040.0f;
  pacc = xfma(pacc, x, 1.0f / 720.0f);
  pacc = xfma(pacc, x, 1.0f / 120.0f);
  pacc = xfma(pacc, x, 1.0f / 24.0f);
  pacc = xfma(pacc, x, 1.0f / 6.0f);
  pacc = xfma(pacc, x, 0.5f);
  pacc = xfma(pacc, x, 1.0f);
  pacc = xfma(pacc, x, 1.0f);
  // exact scaling by 2^k: pacc is in [0.70, 1.42] and |k| <= 60
  return xmul(pacc, ctl_bitsf((uint32_t)(127 + ki) << 23));
}

inline CtlK ctl_consts(double beta1, double beta2, double gamma, double qmin, double qmax,
                       double qsteady_min, double qsteady_max, double qoldinit) {
  CtlK k;
  k.hb1 = (float)(0.5 * beta1);
  k.b2 = (float)beta2;
  k.inv_gamma = (float)(1.0 / gamma);
  k.qmax_inv = (float)(1.0 / qmax);
  k.qmin_inv = (float)(1.0 / qmin);
  k.qmin = (float)qmin;
  k.qs_min = (float)qsteady_min;
  k.qs_max = (float)qsteady_max;
  k.lqoldinit = qoldinit > 0.0 ? ctl_log2f((float)fmax(qoldinit, 1e-30)) : -100.0f;
  return k;
}

// log2 of the mean square, clamped to [-120, 120] (float range of the exponent).
// ms is finite and >= 0 (the callers test finiteness first), so the clamp to
// [2^-120, 2^120] compares bit patterns on the integer pipe.
GBDE_HD float ctl_log2_ms(double ms) {
  const uint64_t lo = 0x3870000000000000ull, hi = 0x4770000000000000ull;  // 2^-120, 2^120
  uint64_t b = mag_bits(ms);
  b = b < lo ? lo : (b > hi ? hi : b);
  double c;
#if defined(__CUDA_ARCH__)
  c = __longlong_as_double((long long)b);
#else
  memcpy(&c, &b, sizeof(c));
#endif
  return ctl_log2f(d2f_rn_bits(c));  // (float)c, off the FP64 pipe
}

// Accepted step: returns r with dt_new = dt * r; updates lqold = log2(qold).
GBDE_HD float ctl_accept(const CtlK& k, double ms, float& lqold) {
  const float L = ctl_log2_ms(ms);
  float ex = xfma(k.hb1, L, -xmul(k.b2, lqold));  // log2(EEst^beta1 / qold^beta2)
  ex = fminf(fmaxf(ex, -60.0f), 60.0f);
  float q = xmul(ctl_exp2f(ex), k.inv_gamma);
  q = fmaxf(k.qmax_inv, fminf(k.qmin_inv, q));
  if (q >= k.qs_min && q <= k.qs_max) q = 1.0f;
  lqold = fmaxf(xmul(0.5f, L), k.lqoldinit);  // log2 max(EEst, qoldinit)
  return 1.0f / q;
}

// Rejected step: returns r with dt_new = dt * r.
GBDE_HD float ctl_reject(const CtlK& k, double ms) {
  if (!isfinite(ms)) return k.qmin;
  float ex = xmul(k.hb1, ctl_log2_ms(ms));
  ex = fminf(fmaxf(ex, -60.0f), 60.0f);
  const float q = fminf(k.qmin_inv, xmul(ctl_exp2f(ex), k.inv_gamma));
  return 1.0f / q;
}

// log2 of a positive finite double over its whole range: the exact binary
// exponent plus ctl_log2f of the mantissa.
GBDE_HD float ctl_log2d(double x) {
  int e;
  const double m = frexp(x, &e);  // exact, m in [0.5, 1)
  return xadd((float)e, ctl_log2f((float)m));
}

// 2^y as a double for |y| up to ~1000 (exact scaling of ctl_exp2f).
GBDE_HD double ctl_exp2d(float y) {
  const float k = rintf(y);
  return ldexp((double)ctl_exp2f(y - k), (int)k);
}

// Hairer-Norsett-Wanner I, Sec. II.4 starting step, from the mean squares of
// the scaled u0 (s0), f(u0) (s1) and of f(u0 + h0 f0) - f0 (s2):
//   d0 = sqrt(s0), d1 = sqrt(s1), h0 = 0.01 d0/d1 (1e-6 if d0 or d1 < 1e-5),
//   d2 = sqrt(s2)/h0, h1 = (0.01/max(d1, d2))^(1/(order+1)),
//   dt = min(100 h0, h1, tspan).
// The powers are evaluated in FP32 through ctl_log2d / ctl_exp2d (a starting
// guess that the controller corrects), identically on host and device.
GBDE_HD double hw_h0(double s0, double s1, double tspan) {
  double h0 = 1e-6;
  if (s0 >= 1e-10 && s1 >= 1e-10 && isfinite(s0) && isfinite(s1))
    h0 = 0.01 * ctl_exp2d(xmul(0.5f, ctl_log2d(s0) - ctl_log2d(s1)));
  return fmin(h0, tspan);
}
GBDE_HD double hw_dt(double h0, double s1, double s2, double tspan, int order) {
  const double d1sq = s1, d2sq = s2 / (h0 * h0);  // squares of d1, d2
  const double msq = fmax(d1sq, d2sq);
  double h1;
  if (!(msq > 1e-30)) {
    h1 = fmax(1e-6, h0 * 1e-3);
  } else if (!isfinite(msq)) {
    h1 = 0.0;  // f overflows at u0 + h0 f0: no usable step (DtLessThanMin)
  } else {
    // log2 h1 = (log2 0.01 - log2 sqrt(msq)) / (order + 1)
    const float lm = xmul(0.5f, ctl_log2d(msq));
    h1 = ctl_exp2d((-6.64385619f - lm) / (float)(order + 1));
  }
  return fmin(fmin(100.0 * h0, h1), tspan);
}

// Reciprocal for the hot loops: a fast hardware estimate refined by one
// Newton-Raphson step r <- r + r (1 - x r) (quadratic convergence: the
// estimate's ~2^-20 relative error becomes ~2^-40; measured on the GPU
// against IEEE division: 9.6e-13).  Its uses -- the error norm's scales, 1/h, the LU
// pivots -- need far less than that, and an IEEE division costs ~10 FP64
// instructions on GB300's narrow FP64 pipe.  x must be finite, normal and
// non-zero; otherwise the result is not finite.
GBDE_HD double rcp64(double x) {
#if defined(__CUDA_ARCH__)
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.0);
  return fma(r, e, r);
#else
  return 1.0 / x;
#endif
}

}  // namespace gbde
