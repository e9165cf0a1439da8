// ff.cuh -- "float-float" numbers: an unevaluated sum hi + lo of two FP32
// values (|lo| <= ulp(hi)/2), about 48 significant bits, built only from FP32
// operations.  GB300 runs FP32 at 61x its FP64 rate, so state, stages and
// right-hand sides in ff cost far fewer FP64-pipe cycles than FP64 while
// keeping near-FP64 accuracy (the FP32-only path cannot: e.g. the Robertson
// rates' cancellation needs more than 24 bits).
//
// Algorithms (error-free transformations):
//   TwoSum (Knuth):        s = a + b, e = (a - (s - bb)) + (b - bb), bb = s - a
//   Fast2Sum (Dekker):     s = a + b, e = b - (s - a)          (|a| >= |b|)
//   TwoProd with FMA:      p = a b, e = fma(a, b, -p)
//   sum:  (a + b) = TwoSum(a.hi, b.hi) + (a.lo + b.lo), renormalised (Fast2Sum)
//   prod: a b     = TwoProd(a.hi, b.hi) + a.hi b.lo + a.lo b.hi, renormalised
// (T.J. Dekker, Numer. Math. 18 (1971) 224-242; D.E. Knuth, TAOCP vol. 2.)
// Only multiplications that the algorithms fuse on purpose use fmaf; the
// TwoSum / Fast2Sum chains contain no products, so FMA contraction cannot
// change them.
#pragma once
#ifndef __CUDACC_RTC__
#include <math.h>
#endif

#include "common.cuh"

namespace gbde {

struct ff {
  float hi, lo;
  ff() = default;
  GBDE_HD constexpr ff(float h, float l) : hi(h), lo(l) {}
  // from a double: hi = rn(d), lo = rn(d - hi)  (folds at compile time for
  // constants; two conversions and one FP64 subtraction at run time)
  GBDE_HD constexpr ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  GBDE_HD constexpr ff(int i) : hi((float)i), lo(0.0f) {}
  GBDE_HD explicit operator double() const { return (double)hi + (double)lo; }
  GBDE_HD explicit operator float() const { return hi + lo; }
};

// Every add / multiply below is a non-contracted IEEE operation (xadd / xmul,
// common.cuh): a product fused into a following add would break the
// error-free transformations.
GBDE_HD ff ff_renorm(float s, float e) {  // Fast2Sum
  const float h = xadd(s, e);
  return ff(h, xadd(e, -xadd(h, -s)));
}

GBDE_HD ff operator+(ff a, ff b) {
  const float s = xadd(a.hi, b.hi);
  const float bb = xadd(s, -a.hi);
  float e = xadd(xadd(a.hi, -xadd(s, -bb)), xadd(b.hi, -bb));
  e = xadd(e, xadd(a.lo, b.lo));
  return ff_renorm(s, e);
}
GBDE_HD ff operator-(ff a) { return ff(-a.hi, -a.lo); }
GBDE_HD ff operator-(ff a, ff b) { return a + (-b); }
GBDE_HD ff operator*(ff a, ff b) {
  const float p = xmul(a.hi, b.hi);
  float e = xfma(a.hi, b.hi, -p);
  e = xfma(a.hi, b.lo, xfma(a.lo, b.hi, e));
  return ff_renorm(p, e);
}
GBDE_HD ff& operator+=(ff& a, ff b) { return a = a + b; }
GBDE_HD ff& operator-=(ff& a, ff b) { return a = a - b; }
GBDE_HD ff& operator*=(ff& a, ff b) { return a = a * b; }
GBDE_HD bool operator<(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

// a pair is finite iff its leading part is
GBDE_HD bool val_finite(ff x) { return isfinite(x.hi); }
// a pair rounded to FP32: hi + lo in one correctly rounded FP32 addition
// (the exact sum rounded once; the FP64 route rounds twice)
GBDE_HD float val_f32(ff x) { return xadd(x.hi, x.lo); }

template <class T> struct is_ff { static constexpr bool value = false; };
template <> struct is_ff<ff> { static constexpr bool value = true; };

}  // namespace gbde
