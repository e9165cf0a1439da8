// philox.h -- Philox4x32-10 counter-based generator and a host/device
// bit-identical normal transform.
//
// Replaces the `rng` kwarg machinery of the reference's noise processes
// (get_rng / set_rng! / supports_solve_rng, test/qa/qa.jl:152,189,196;
// NoiseProblem qa.jl:77).  The stream of normals of trajectory `traj` under
// key `seed` is a pure function of (seed, traj, draw index), so any
// trajectory's Brownian path can be regenerated on the host.
//
// Philox4x32-10: J.K. Salmon, M.A. Moraes, R.O. Dror, D.E. Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11.  Round: (hi0,lo0) = M0*c0,
// (hi1,lo1) = M1*c2, c <- (hi1^c1^k0, lo1, hi0^c3^k1, lo0); the key is bumped
// by the Weyl constants (W0, W1) between rounds.
//
// Normal transform: Box-Muller (G.E.P. Box, M.E. Muller, Ann. Math. Stat. 29
// (1958) 610-611).  Its log and sin/cos are this file's own series
// evaluations, built only from correctly rounded IEEE operations (explicit
// non-contracted multiply/add/fma, division, sqrt), so the host and the
// device produce identical bits:
//   log x = e ln2 + 2 atanh(s), s = (m-1)/(m+1), x = m 2^e, m in [1/sqrt2, sqrt2)
//   (atanh series s + s^3/3 + s^5/5 + ...);
//   sin / cos of 2 pi u: exact quadrant reduction of 4u, then the Taylor
//   series of sin r, cos r for |r| <= pi/4.
// Host code that includes this header must be compiled with
// -ffp-contract=off.
#pragma once
#ifndef __CUDACC_RTC__
#include <stdint.h>
#include <math.h>
#endif
#include "common.cuh"

namespace gbde {

struct Philox4 {
  uint32_t x, y, z, w;
};

GBDE_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  lo = a * b;
  hi = __umulhi(a, b);
#else
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
#endif
}

GBDE_HD Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(M0, c.x, hi0, lo0);
    mulhilo32(M1, c.z, hi1, lo1);
    c = Philox4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

template <class T> struct BMConst;
template <> struct BMConst<double> {
  static constexpr int NLOG = 12;   // atanh terms: s^2 <= 0.0295, 0.0295^12 < 1e-18
  static constexpr int NTRIG = 9;   // Taylor terms for |r| <= pi/4
  static constexpr double ln2_hi = 0.6931471805599453;     // ln 2 rounded to double
  static constexpr double ln2_lo = 2.3190468138462996e-17; // ln 2 - ln2_hi
  static constexpr double pio2_hi = 1.5707963267948966;    // pi/2 rounded
  static constexpr double pio2_lo = 6.123233995736766e-17; // pi/2 - pio2_hi
  static constexpr double sqrt_half = 0.7071067811865476;
};
template <> struct BMConst<float> {
  static constexpr int NLOG = 6;
  static constexpr int NTRIG = 5;
  static constexpr float ln2_hi = 0.693147182f;
  static constexpr float ln2_lo = -1.90465421e-09f;
  static constexpr float pio2_hi = 1.57079637f;
  static constexpr float pio2_lo = -4.37113883e-08f;
  static constexpr float sqrt_half = 0.707106781f;
};

// log(x) for a normal positive x (x in (0, 1] here).
template <class T>
GBDE_HD T bm_log(T x) {
  using C = BMConst<T>;
  int e;
  T m = frexp(x, &e);  // x = m 2^e, m in [0.5, 1): exact
  if (m < C::sqrt_half) {
    m = m + m;  // exact
    e -= 1;
  }
  const T s = (m - T(1)) / (m + T(1));  // m - 1 is exact (Sterbenz); IEEE division
  const T s2 = xmul(s, s);
  // P(s2) = sum_{k>=0} s2^k / (2k+1), Horner from the highest term
  T pacc = T(1) / T(2 * C::NLOG + 1);
#pragma unroll
  for (int k = C::NLOG - 1; k >= 0; --k) pacc = xfma(pacc, s2, T(1) / T(2 * k + 1));
  const T lm = xmul(xadd(s, s), pacc);  // 2 s P
  const T fe = (T)e;
  return xadd(xfma(fe, C::ln2_hi, lm), xmul(fe, C::ln2_lo));
}

// (cos(2 pi u), sin(2 pi u)) for u in [0, 1).
template <class T>
GBDE_HD void bm_sincos2pi(T u, T& co, T& si) {
  using C = BMConst<T>;
  const T v = u * T(4);  // exact (power of two)
  T qf = floor(v);
  T f = v - qf;          // exact, in [0, 1)
  int q = (int)qf;
  if (f > T(0.5)) {      // center: f in [-1/2, 1/2]
    f = f - T(1);
    q += 1;
  }
  q &= 3;
  const T r = xfma(f, C::pio2_hi, xmul(f, C::pio2_lo));  // f pi/2, |r| <= pi/4
  const T r2 = xmul(r, r);
  // sin r = r (1 - r2/3! + r2^2/5! - ...), cos r = 1 - r2/2! + ...
  T sp = T(0), cp = T(0);
  {
    // coefficients (-1)^k / (2k+1)! and (-1)^k / (2k)!, built by division
    T sc[BMConst<T>::NTRIG + 1], cc[BMConst<T>::NTRIG + 1];
    T fs = T(1), fc = T(1);
#pragma unroll
    for (int k = 0; k <= C::NTRIG; ++k) {
      sc[k] = ((k & 1) ? T(-1) : T(1)) / fs;
      cc[k] = ((k & 1) ? T(-1) : T(1)) / fc;
      fs = fs * T((2 * k + 2) * (2 * k + 3));
      fc = fc * T((2 * k + 1) * (2 * k + 2));
    }
    sp = sc[C::NTRIG];
    cp = cc[C::NTRIG];
#pragma unroll
    for (int k = C::NTRIG - 1; k >= 0; --k) {
      sp = xfma(sp, r2, sc[k]);
      cp = xfma(cp, r2, cc[k]);
    }
  }
  const T sr = xmul(r, sp), cr = cp;
  switch (q) {
    case 0: co = cr; si = sr; break;
    case 1: co = -sr; si = cr; break;
    case 2: co = -cr; si = -sr; break;
    default: co = sr; si = -cr; break;
  }
}

// Box-Muller pair from two uniforms u1 in (0, 1], u2 in [0, 1).
template <class T>
GBDE_HD void box_muller(T u1, T u2, T& z0, T& z1) {
  const T r = sqrt(xmul(T(-2), bm_log(u1)));
  T c, s;
  bm_sincos2pi(u2, c, s);
  z0 = xmul(r, c);
  z1 = xmul(r, s);
}

// ---- the per-trajectory normal stream
// FP64: normals 2b, 2b+1 come from Philox block b (53-bit uniforms from
// (x,y) and (z,w)).  FP32: normals 4b..4b+3 from block b (24-bit uniforms).
// Counter = (b_lo, b_hi, traj_lo, traj_hi), key = (seed_lo, seed_hi).
GBDE_HD Philox4 philox_block(uint64_t seed, uint64_t traj, uint64_t b) {
  return philox4x32_10(Philox4{(uint32_t)b, (uint32_t)(b >> 32), (uint32_t)traj,
                               (uint32_t)(traj >> 32)},
                       (uint32_t)seed, (uint32_t)(seed >> 32));
}

GBDE_HD void philox_normal_pair_f64(uint64_t seed, uint64_t traj, uint64_t b, double& z0,
                                    double& z1) {
  const Philox4 r = philox_block(seed, traj, b);
  const uint64_t a = ((uint64_t)(r.x >> 5) << 26) | (uint64_t)(r.y >> 6);  // 53 bits
  const uint64_t c = ((uint64_t)(r.z >> 5) << 26) | (uint64_t)(r.w >> 6);
  const double u1 = ((double)a + 0.5) * 1.1102230246251565e-16;  // (a + 1/2) 2^-53 in (0,1)
  const double u2 = (double)c * 1.1102230246251565e-16;          // [0, 1)
  box_muller(u1, u2, z0, z1);
}

GBDE_HD void philox_normal_quad_f32(uint64_t seed, uint64_t traj, uint64_t b, float* z) {
  const Philox4 r = philox_block(seed, traj, b);
  const float s = 5.9604644775390625e-08f;  // 2^-24
  const float u1 = ((float)(r.x >> 8) + 0.5f) * s;
  const float u2 = (float)(r.y >> 8) * s;
  const float u3 = ((float)(r.z >> 8) + 0.5f) * s;
  const float u4 = (float)(r.w >> 8) * s;
  box_muller(u1, u2, z[0], z[1]);
  box_muller(u3, u4, z[2], z[3]);
}

GBDE_HD double philox_normal_f64(uint64_t seed, uint64_t traj, uint64_t d) {
  double z0, z1;
  philox_normal_pair_f64(seed, traj, d >> 1, z0, z1);
  return (d & 1) ? z1 : z0;
}

GBDE_HD float philox_normal_f32(uint64_t seed, uint64_t traj, uint64_t d) {
  float z[4];
  philox_normal_quad_f32(seed, traj, d >> 2, z);
  return z[d & 3];
}

}  // namespace gbde
