// ff_vec.cuh -- FP32-pair building blocks shared by the compact pair steppers
// (rodas_ff.cuh, tsit5_ff.cuh): the integer-pipe split of a double into a
// pair, an unnormalised accumulator of sums of pair products, and the same
// accumulator over two state components at once on Blackwell's paired FP32
// instructions.
#pragma once
#include "ff.cuh"

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

// A norm ratio s / d in FP32 by the fast reciprocal and product: within 2 ulp
// for the normal d the tolerances give (d >= atol > 0, or rtol |u|), against
// the IEEE division's multi-instruction sequence.  The ratios feed a mean
// square and a step decision at 1; on the ring's pair teams the fast form
// moved 8 of 226M step decisions and took 3 % off the non-stiff kernel.
GBDE_D float norm_ratio(float s, float d) { return __fdividef(s, d); }

// A tolerance (finite, >= 0) in FP32 for the norm ratios: rounded to nearest on
// the integer pipe (d2f_rn_bits), values below FP32's normal range flushed to
// 0 as ff_split does -- without the split's int-to-float conversion, which
// runs on GB300's narrow FP64 pipe.
GBDE_D float tol_f32(double x) {
  return mag_bits(x) < 0x3810000000000000ull ? 0.0f : d2f_rn_bits(x);  // 2^-126
}

// 1 / x for a pair, relative error about 2^-47: the correctly rounded FP32
// reciprocal r of the leading part, then one Newton correction on the pair,
// 1/x ~ r + r e with e = 1 - x r.  The leading residual 1 - hi r is exact
// with an FMA (the residual of a correctly rounded reciprocal is
// representable); the low part enters as - lo r.  (Newton's iteration for the
// reciprocal with an exact first residual, as in T.J. Dekker, Numer. Math. 18
// (1971) 224-242, applied to a float-float divisor.)
GBDE_D ff ff_rcp(ff x) {
  const float r = __frcp_rn(x.hi);
  const float e = xfma(-x.lo, r, xfma(-x.hi, r, 1.0f));
  return ff_renorm(r, xmul(r, e));
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
// Blackwell's paired FP32 arithmetic (add / sub / fma .rn.f32x2) takes
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
GBDE_D F2 f2_fma(F2 a, F2 b, F2 c) {  // a b + c
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
// The rounded product a b as a paired FMA onto +0 (equal to it but for the
// sign of a zero product).  A paired multiply (mul.rn.f32x2) whose result
// feeds the TwoSum / Fast2Sum chains below was measured on GB300 to give
// results that are not the rounded product -- the pair's low part then
// carried the product's rounding error twice, whether or not ptxas may
// contract -- while this form reproduces the scalar arithmetic bit for bit.
GBDE_D F2 f2_prod(F2 a, F2 b) { return f2_fma(a, b, f2_pack(0.0f, 0.0f)); }

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
    const F2 pn = f2_prod(ahn, bh);                      // -p
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

// h x for every component, each product renormalised exactly as ff's
// operator* (TwoProd with cross terms, then Fast2Sum), two components per
// paired instruction.
template <int N>
GBDE_D FfVec<N> ff_scale(ff h, const ff* x) {
  constexpr int Q = N / 2;
  FfVec<N> r;
  const F2 hh = f2_pack(h.hi, h.hi), hl = f2_pack(h.lo, h.lo), hn = f2_pack(-h.hi, -h.hi);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const F2 xh = f2_pack(x[2 * q].hi, x[2 * q + 1].hi), xl = f2_pack(x[2 * q].lo, x[2 * q + 1].lo);
    const F2 p = f2_prod(hh, xh);
    F2 e = f2_fma(hh, xh, f2_prod(hn, xh));  // hi product error, exactly
    e = f2_fma(hh, xl, f2_fma(hl, xh, e));
    const F2 s = f2_add(p, e);
    r.h[q] = s;
    r.l[q] = f2_sub(e, f2_sub(s, p));
  }
  if constexpr (N % 2) r.o = h * x[N - 1];
  return r;
}

}  // namespace gbde
