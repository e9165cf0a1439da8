// common.cuh -- host/device helpers shared by every solver kernel.
#pragma once
// Under NVRTC (runtime-compiled user models, rtc.cu) there are no C library
// headers: the runtime-compiled source defines the fixed-width integer types
// itself, and the math functions are NVRTC built-ins.
#ifndef __CUDACC_RTC__
#include <stdint.h>
#include <string.h>
#include <math.h>
#endif

#if defined(__CUDACC__)
#define GBDE_HD __host__ __device__ __forceinline__
#define GBDE_D __device__ __forceinline__
#else
#define GBDE_HD inline
#define GBDE_D inline
#endif

namespace gbde {

template <class T> GBDE_HD T tmax(T a, T b) { return a > b ? a : b; }
template <class T> GBDE_HD T tmin(T a, T b) { return a < b ? a : b; }
template <class T> GBDE_HD T tabs(T a) { return a < T(0) ? -a : a; }

GBDE_HD bool finite_d(double x) { return isfinite(x); }

// ---- non-contracted arithmetic (identical rounding on host and device)
#if defined(__CUDA_ARCH__)
GBDE_HD double xmul(double a, double b) { return __dmul_rn(a, b); }
GBDE_HD double xadd(double a, double b) { return __dadd_rn(a, b); }
GBDE_HD double xfma(double a, double b, double c) { return __fma_rn(a, b, c); }
GBDE_HD float xmul(float a, float b) { return __fmul_rn(a, b); }
GBDE_HD float xadd(float a, float b) { return __fadd_rn(a, b); }
GBDE_HD float xfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
GBDE_HD double xmul(double a, double b) { return a * b; }
GBDE_HD double xadd(double a, double b) { return a + b; }
GBDE_HD double xfma(double a, double b, double c) { return fma(a, b, c); }
GBDE_HD float xmul(float a, float b) { return a * b; }
GBDE_HD float xadd(float a, float b) { return a + b; }
GBDE_HD float xfma(float a, float b, float c) { return fmaf(a, b, c); }
#endif

// x as an ordered integer: for non-NaN doubles (either sign),
// ord_bits(a) <= ord_bits(b) iff a <= b.  Comparisons on the integer pipe.
GBDE_HD uint64_t ord_bits(double x) {
#if defined(__CUDA_ARCH__)
  const uint64_t b = (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
#endif
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// |x| as an ordered integer: for non-NaN doubles, mag_bits(a) < mag_bits(b)
// iff |a| < |b|.  Compares on the integer pipe instead of the FP64 pipe.
GBDE_HD uint64_t mag_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x) & 0x7fffffffffffffffull;
#else
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
  return b & 0x7fffffffffffffffull;
#endif
}

// float -> double widening on the integer pipe (the conversion instruction runs
// on GB300's narrow FP64 pipe): exact for normal floats, infinities and NaN;
// zeros and subnormal floats give a signed zero.
GBDE_HD double f2d_bits(float x) {
  uint32_t b;
#if defined(__CUDA_ARCH__)
  b = __float_as_uint(x);
#else
  memcpy(&b, &x, sizeof(b));
#endif
  const uint32_t e = (b >> 23) & 0xffu, s = b & 0x80000000u, m = b & 0x7fffffu;
  const uint32_t ed = e == 0u ? 0u : (e == 0xffu ? 0x7ffu : e + 896u);
  const uint32_t hw = s | (ed << 20) | (e == 0u ? 0u : (m >> 3));
  const uint32_t lw = e == 0u ? 0u : (m << 29);
#if defined(__CUDA_ARCH__)
  return __hiloint2double((int)hw, (int)lw);
#else
  const uint64_t v = ((uint64_t)hw << 32) | lw;
  double d;
  memcpy(&d, &v, sizeof(d));
  return d;
#endif
}

// An FP64 value carried as its bit pattern: a driver loop's copies and selects
// of it stay on the integer pipe (GB300 runs FP64 moves on its narrow FP64
// pipe); reading it as a double is a reinterpretation.
struct F64Bits {
  uint64_t b;
  F64Bits() = default;
  GBDE_HD F64Bits(double x) {
#if defined(__CUDA_ARCH__)
    b = (uint64_t)__double_as_longlong(x);
#else
    memcpy(&b, &x, sizeof(b));
#endif
  }
  GBDE_HD operator double() const {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof(x));
    return x;
#endif
  }
};

// double -> float, rounded to nearest even, on the integer pipe: the value the
// conversion instruction gives (that one runs on GB300's narrow FP64 pipe),
// for finite x whose float is normal (2^-126 <= |x| < 2^128 after rounding).
GBDE_HD float d2f_rn_bits(double x) {
  uint64_t b;
#if defined(__CUDA_ARCH__)
  b = (uint64_t)__double_as_longlong(x);
#else
  memcpy(&b, &x, sizeof(b));
#endif
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const uint32_t e = (uint32_t)((b >> 52) & 0x7ffu) - 896u;  // float's biased exponent
  const uint32_t rest = (uint32_t)b & 0x1fffffffu;           // the 29 bits dropped
  uint32_t f = (e << 23) | (uint32_t)((b >> 29) & 0x7fffffu);
  // a carry out of the significand moves into the exponent, as it should
  f += (rest > 0x10000000u || (rest == 0x10000000u && (f & 1u))) ? 1u : 0u;
  f |= sign;
#if defined(__CUDA_ARCH__)
  return __uint_as_float(f);
#else
  float r;
  memcpy(&r, &f, sizeof(r));
  return r;
#endif
}

// Finiteness of a state component: through the FP64 value for double and
// float; the pair type (ff.cuh) overloads it with a test of its leading part.
template <class T>
GBDE_HD bool val_finite(T x) {
  return isfinite((double)x);
}
// FP32 values test directly: no conversion on the FP64 pipe
GBDE_HD bool val_finite(float x) { return isfinite(x); }

// A state component rounded to FP32 for the FP32 output; the pair type
// (ff.cuh) overloads it with one rounding of hi + lo.
template <class T>
GBDE_HD float val_f32(T x) {
  return (float)x;
}

// TwoSum in the working precision T (the FP32 path keeps its state as an
// unevaluated sum hi + lo so that rounding does not accumulate over steps).
template <class T>
GBDE_HD void two_sum_t(T a, T b, T& s, T& e) {
  s = a + b;
  T bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

}  // namespace gbde
