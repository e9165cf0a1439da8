// common.cuh -- host/device helpers shared by every solver kernel.
#pragma once
#include <stdint.h>
#include <math.h>

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

// Error-free sum (Knuth TwoSum): s + e == a + b exactly.  Used for the
// compensated time accumulation of the mixed-precision path.
GBDE_HD void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// TwoSum in the working precision T (the FP32 path keeps its state as an
// unevaluated sum hi + lo so that rounding does not accumulate over steps).
template <class T>
GBDE_HD void two_sum_t(T a, T b, T& s, T& e) {
  s = a + b;
  T bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Compensated time: t = hi + lo.
struct CTime {
  double hi, lo;
  GBDE_HD double value() const { return hi + lo; }
  GBDE_HD void add(double dt) {
    double s, e;
    two_sum(hi, dt, s, e);
    e += lo;
    hi = s + e;
    lo = e - (hi - s);
  }
};

}  // namespace gbde
