// summary.cu -- ensemble statistics on the device: per save point and
// component, the mean, the variance and quantiles across trajectories.
//
// Replaces SciMLBase's EnsembleSummary / EnsembleAnalysis
// (timepoint_meanvar, timepoint_quantile; EnsembleSummary and
// EnsembleAnalysis, test/qa/qa.jl:54,211) for solutions that stay in device
// memory: a caller that only needs the statistics reads back
// n_save * n_state * (2 + n_quantiles) numbers instead of the whole ensemble.
//
// Definitions (as Julia's Statistics and numpy's defaults):
//   mean = sum x / N;  var = sum (x - mean)^2 / (N - 1)  (NaN for N = 1);
//   quantile q: h = (N - 1) q, k = floor(h), the k-th and (k+1)-th order
//   statistics a <= b (0-based) interpolated linearly with gamma = h - k
//   (numpy's lerp: a + (b - a) gamma, or b - (b - a)(1 - gamma) for
//   gamma >= 1/2).  A column that holds a NaN (a save slot of a failed
//   trajectory) has NaN mean, variance and quantiles.
//
// Kernels, all HBM-bound on u[N][C] (C = n_save * n_state):
//  1. k_sum: per-thread shifted sums S1 = sum (x - s), S2 = sum (x - s)^2
//     with s = u[0][c]; the grid stride is a multiple of C, so a thread always
//     sees the same column.  Per-CTA partials, reduced in a fixed order by
//     k_sum_final (deterministic, no floating-point atomics).
//  2. k_keys: u -> column-major ordered keys keys[c][i] (the value's bits
//     mapped so that unsigned order = numeric order).
//  3. radix selection of every target rank (2 per quantile) at once: per
//     8-bit digit, k_digit_hist counts the digits of the keys that match each
//     target's prefix (a shared-memory histogram per target, merged with one
//     global atomic per non-zero bin), and k_digit_pick moves each target to
//     the bin that holds its rank.  After sizeof(key) passes every target is
//     an exact order statistic.
//  4. k_quantiles interpolates.
#include <cstdio>
#include <cstring>
#include <utility>

#include <cuda_runtime.h>

#include "../../include/gbde.h"
#include "launch.h"

namespace gbde {

namespace {

constexpr int kMaxTargets = 2 * GBDE_SUMMARY_MAX_Q;
constexpr int kBins = 256;

__device__ __forceinline__ uint32_t ord_key(float x) {
  const uint32_t b = __float_as_uint(x);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ uint64_t ord_key(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_value(uint32_t k) {
  const uint32_t b = (k >> 31) ? (k & 0x7fffffffu) : ~k;
  return (double)__uint_as_float(b);
}
__device__ __forceinline__ double key_value(uint64_t k) {
  const uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

// Shifted sums of one value into (S1, S2).  FP64 values accumulate in FP64.
// FP32 values accumulate on the FP32 pipe as compensated pairs (Neumaier sums
// of the exact difference x - s and of its square), because GB300's FP64
// pipe would otherwise bound this HBM-streaming pass: each pair sum is within
// a few FP32 ulps squared of exact, far below the FP64 combination error.
struct SumAcc64 {
  double s1 = 0.0, s2 = 0.0;
  __device__ __forceinline__ void add(double x, double s) {
    const double d = x - s;
    s1 += d;
    s2 += d * d;
  }
  __device__ __forceinline__ double v1() const { return s1; }
  __device__ __forceinline__ double v2() const { return s2; }
};
struct SumAcc32 {
  float a1 = 0.f, c1 = 0.f, a2 = 0.f, c2 = 0.f;
  // Neumaier: a += x with the rounding error collected in c
  __device__ __forceinline__ static void nadd(float& a, float& c, float x) {
    const float t = __fadd_rn(a, x);
    c = __fadd_rn(c, fabsf(a) >= fabsf(x) ? __fadd_rn(__fadd_rn(a, -t), x)
                                          : __fadd_rn(__fadd_rn(x, -t), a));
    a = t;
  }
  __device__ __forceinline__ void add(float x, float s) {
    // d = x - s exactly as dh + dl (TwoSum)
    const float dh = __fadd_rn(x, -s);
    const float bb = __fadd_rn(dh, -x);
    const float dl = __fadd_rn(__fadd_rn(x, -__fadd_rn(dh, -bb)), __fadd_rn(-s, -bb));
    nadd(a1, c1, dh);
    c1 = __fadd_rn(c1, dl);
    // d^2 = p + e (TwoProd of dh, plus 2 dh dl; dl^2 is below FP32 resolution)
    const float p = __fmul_rn(dh, dh);
    const float e = __fmaf_rn(__fmul_rn(2.0f, dh), dl, __fmaf_rn(dh, dh, -p));
    nadd(a2, c2, p);
    c2 = __fadd_rn(c2, e);
  }
  __device__ __forceinline__ double v1() const { return (double)a1 + (double)c1; }
  __device__ __forceinline__ double v2() const { return (double)a2 + (double)c2; }
};
template <class T> struct SumAccOf;
template <> struct SumAccOf<double> { using type = SumAcc64; };
template <> struct SumAccOf<float> { using type = SumAcc32; };

template <class T>
__global__ void __launch_bounds__(256) k_sum(const T* __restrict__ u, int64_t total, int C,
                                             double* __restrict__ partial) {
  // stride = gridDim.x * blockDim.x is a multiple of C: column fixed per thread
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = (int)(start % C);
  const T s = u[c];
  typename SumAccOf<T>::type acc;
  for (int64_t e = start; e < total; e += stride) acc.add(u[e], s);
  // per-CTA column sums in a fixed order: thread j holds column (base + j) % C
  extern __shared__ double sh[];  // [blockDim][2]
  sh[2 * threadIdx.x] = acc.v1();
  sh[2 * threadIdx.x + 1] = acc.v2();
  __syncthreads();
  double* out = partial + (size_t)blockIdx.x * C * 2;
  const int64_t base = (int64_t)blockIdx.x * blockDim.x;
  for (int t = threadIdx.x; t < C; t += blockDim.x) {
    double a = 0.0, b = 0.0;
    const int first = (int)(((int64_t)t - base % C + C) % C);
    for (int j = first; j < (int)blockDim.x; j += C) {
      a += sh[2 * j];
      b += sh[2 * j + 1];
    }
    out[2 * t] = a;
    out[2 * t + 1] = b;
  }
}

// One warp per column: lane l sums the partials of blocks l, l + 32, ...;
// the butterfly then combines the lanes in a fixed order (deterministic).
template <class T>
__global__ void __launch_bounds__(256) k_sum_final(const T* __restrict__ u,
                                                   const double* __restrict__ partial, int nblk,
                                                   int C, int64_t N, double* __restrict__ mean,
                                                   double* __restrict__ var,
                                                   double* __restrict__ mean_scratch) {
  const int lane = threadIdx.x & 31;
  const int c = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (c >= C) return;
  double s1 = 0.0, s2 = 0.0;
  for (int b = lane; b < nblk; b += 32) {
    s1 += partial[((size_t)b * C + c) * 2];
    s2 += partial[((size_t)b * C + c) * 2 + 1];
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if (lane != 0) return;
  const double s = (double)u[c];
  const double m = s + s1 / (double)N;
  const double v = N > 1 ? fmax(s2 - s1 * s1 / (double)N, 0.0) / (double)(N - 1)
                         : __longlong_as_double(0x7ff8000000000000ll);
  const bool nan = isnan(s1) || isnan(s2);
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  if (mean) mean[c] = nan ? qnan : m;
  if (var) var[c] = nan ? qnan : v;
  mean_scratch[c] = nan ? qnan : m;
}

// u[N][C] -> keys[C][N] through a 32 x 32 shared-memory tile: reads
// coalesced along c, writes coalesced along i.  Block 32 x 8 threads.
template <class T, class K>
__global__ void __launch_bounds__(256) k_keys(const T* __restrict__ u, int64_t N, int C,
                                              int64_t pitch, K* __restrict__ keys) {
  __shared__ K tile[32][33];
  const int ntc = (C + 31) / 32;
  const int64_t ntr = (N + 31) / 32;
  for (int64_t b = blockIdx.x; b < ntr * ntc; b += gridDim.x) {
    const int64_t i0 = (b / ntc) * 32;
    const int c0 = (int)(b % ntc) * 32;
    for (int r = threadIdx.y; r < 32; r += 8) {
      const int64_t i = i0 + r;
      const int c = c0 + threadIdx.x;
      if (i < N && c < C) tile[r][threadIdx.x] = ord_key(u[i * C + c]);
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
      const int c = c0 + r;
      const int64_t i = i0 + threadIdx.x;
      if (i < N && c < C) keys[(size_t)c * pitch + i] = tile[threadIdx.x][r];
    }
    __syncthreads();
  }
}

// Per target (c, t): prefix of the key digits fixed so far and the rank
// still to find inside it.
struct Target {
  unsigned long long prefix;
  long long rank;
};

// Targets with equal prefixes share one histogram, kept under the first of
// them (the "leader"); a key matches at most one leader's prefix, so each key
// is counted once.  A column's keys concentrate on few leading digits, so
// plain per-key atomics would serialise: each thread counts runs of equal
// (leader, digit) in registers, and the CTA's 8 warps spread over kSub
// sub-histograms.
constexpr int kSub = 4;

template <class K>
__global__ void __launch_bounds__(256) k_digit_hist(const K* __restrict__ keys, int64_t N,
                                                    int64_t pitch, int C, int T, int pass,
                                                    const Target* __restrict__ tg,
                                                    unsigned* __restrict__ hist) {
  // blockIdx.y = column; the x blocks split its N keys
  extern __shared__ unsigned h[];  // [kSub][T][kBins]
  __shared__ unsigned long long pre[kMaxTargets];
  __shared__ int leader[kMaxTargets];
  __shared__ int nlead;
  const int c = blockIdx.y;
  constexpr int BITS = 8 * (int)sizeof(K);
  const int shift = BITS - 8 * (pass + 1);
  for (int i = threadIdx.x; i < kSub * T * kBins; i += blockDim.x) h[i] = 0;
  if (threadIdx.x < T) pre[threadIdx.x] = tg[(size_t)c * T + threadIdx.x].prefix;
  __syncthreads();
  if (threadIdx.x == 0) {
    int n = 0;
    for (int t = 0; t < T; ++t) {
      bool first = true;
      for (int q = 0; q < t; ++q) first = first && pre[q] != pre[t];
      if (first) leader[n++] = t;
    }
    nlead = n;
  }
  __syncthreads();
  const int nl = nlead;
  unsigned* hs = h + (size_t)((threadIdx.x >> 5) % kSub) * T * kBins;
  const K* col = keys + (size_t)c * pitch;
  // run-length count in registers: a thread's successive keys mostly share
  // their (leader, digit) slot, so the shared histogram sees one atomic per
  // run instead of one per key
  int run_slot = -1;
  unsigned run = 0;
  // 16-byte loads (the column pitch is a multiple of 16 bytes): more bytes in
  // flight per thread than one key per iteration
  constexpr int V = 16 / (int)sizeof(K);
  using Vec = uint4;
  const int64_t nvec = (N + V - 1) / V;
  const Vec* cv = reinterpret_cast<const Vec*>(col);
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvec;
       v += (int64_t)gridDim.x * blockDim.x) {
    const Vec w = __ldg(cv + v);
    const K* kk = reinterpret_cast<const K*>(&w);
#pragma unroll
    for (int j = 0; j < V; ++j) {
      if (v * V + j >= N) break;
      const K k = kk[j];
      const unsigned digit = (unsigned)((k >> shift) & 0xffu);
      int hit = -1;
      if (pass == 0) {
        hit = 0;  // every target has the empty prefix
      } else {
        const unsigned long long hi = (unsigned long long)(k >> (shift + 8));
        for (int q = 0; q < nl; ++q)
          if (hi == pre[leader[q]]) hit = leader[q];
      }
      if (hit < 0) continue;
      const int slot = hit * kBins + (int)digit;
      if (slot == run_slot) {
        ++run;
      } else {
        if (run) atomicAdd(&hs[run_slot], run);
        run_slot = slot;
        run = 1;
      }
    }
  }
  if (run) atomicAdd(&hs[run_slot], run);
  __syncthreads();
  unsigned* g = hist + (size_t)c * kMaxTargets * kBins;
  for (int i = threadIdx.x; i < T * kBins; i += blockDim.x) {
    unsigned v = 0;
    for (int q = 0; q < kSub; ++q) v += h[(size_t)q * T * kBins + i];
    if (v) atomicAdd(&g[i], v);
  }
}

// One thread per (column, target): walk its leader's bins to the one holding
// the rank.  Reads tin, writes tout (the leader lookup reads other targets'
// prefixes, so the update cannot be in place).
__global__ void k_digit_pick(int C, int T, int pass, const Target* __restrict__ tin,
                             Target* __restrict__ tout, const unsigned* __restrict__ hist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C * T) return;
  const int c = i / T, t = i % T;
  Target x = tin[i];
  int lead = t;
  for (int q = t - 1; q >= 0; --q)
    if (tin[(size_t)c * T + q].prefix == x.prefix) lead = q;
  const unsigned* h = hist + ((size_t)c * kMaxTargets + lead) * kBins;
  long long r = x.rank;
  int d = 0;
  for (; d < kBins - 1; ++d) {
    if (r < (long long)h[d]) break;
    r -= h[d];
  }
  x.prefix = (x.prefix << 8) | (unsigned long long)d;
  x.rank = r;
  tout[i] = x;
}

__global__ void k_clear(unsigned* __restrict__ p, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = 0u;
}

__global__ void k_targets_init(int C, int nq, const double* __restrict__ q, int64_t N,
                               Target* __restrict__ tg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int T = 2 * nq;
  if (i >= C * T) return;
  const int t = i % T, j = t / 2;
  const double h = (double)(N - 1) * q[j];
  long long k = (long long)floor(h);
  if (k > N - 1) k = N - 1;
  long long r = k + (t & 1);
  if (r > N - 1) r = N - 1;
  tg[i].prefix = 0ull;
  tg[i].rank = r;
}

template <class K>
__global__ void k_quantiles(int C, int nq, const double* __restrict__ q, int64_t N,
                            const Target* __restrict__ tg, const double* __restrict__ mean,
                            double* __restrict__ qv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C * nq) return;
  const int c = i / nq, j = i % nq;
  const int T = 2 * nq;
  const double a = key_value((K)tg[(size_t)c * T + 2 * j].prefix);
  const double b = key_value((K)tg[(size_t)c * T + 2 * j + 1].prefix);
  const double h = (double)(N - 1) * q[j];
  const double g = h - floor(h);
  const double diff = b - a;
  double r = g >= 0.5 ? b - diff * (1.0 - g) : a + diff * g;
  if (isnan(mean[c])) r = __longlong_as_double(0x7ff8000000000000ll);
  qv[(size_t)j * C + c] = r;
}

}  // namespace

size_t summary_scratch_bytes(int64_t N, int C, int u_f32, int nq, int sum_blocks) {
  size_t b = (size_t)sum_blocks * C * 2 * sizeof(double) + (size_t)C * sizeof(double);
  if (nq > 0) {
    b += (size_t)((N + 7) & ~(int64_t)7) * C * (u_f32 ? 4 : 8);
    b += (size_t)C * kMaxTargets * kBins * sizeof(unsigned);
    b += 2 * (size_t)C * 2 * nq * sizeof(Target);
    b += 16 * sizeof(double);
  }
  return b + 8 * 256;  // each of the (at most 7) sub-buffers is rounded up to 256 B
}

int summary_sum_blocks(int C, int num_sms) {
  int g = 1;
  int a = C, b = 256;  // g * 256 must be a multiple of C: g = multiple of C / gcd(C, 256)
  while (b) {
    const int t = a % b;
    a = b;
    b = t;
  }
  const int unit = C / a;
  const int want = 4 * num_sms;
  g = unit * ((want + unit - 1) / unit);
  return g;
}

// Enqueue the statistics of u[N][C] (device) on stream s; every output is
// device memory and may be NULL.  scratch holds summary_scratch_bytes(...).
cudaError_t enqueue_summary(const void* u, int u_f32, int64_t N, int C, int nq,
                            const double* q_host, double* mean, double* var, double* qv,
                            void* scratch, int num_sms, cudaStream_t s) {
  const int nblk = summary_sum_blocks(C, num_sms);
  char* p = static_cast<char*>(scratch);
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  double* partial = (double*)take((size_t)nblk * C * 2 * sizeof(double));
  double* mscr = (double*)take((size_t)C * sizeof(double));
  if (u_f32)
    k_sum<float><<<nblk, 256, 256 * 2 * sizeof(double), s>>>((const float*)u, N * C, C, partial);
  else
    k_sum<double><<<nblk, 256, 256 * 2 * sizeof(double), s>>>((const double*)u, N * C, C, partial);
  const int g1 = (C * 32 + 255) / 256;
  if (u_f32)
    k_sum_final<float><<<g1, 256, 0, s>>>((const float*)u, partial, nblk, C, N, mean, var, mscr);
  else
    k_sum_final<double><<<g1, 256, 0, s>>>((const double*)u, partial, nblk, C, N, mean, var, mscr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nq == 0 || qv == nullptr) return e;

  const int T = 2 * nq;
  const int64_t pitch = (N + 7) & ~(int64_t)7;  // 16-byte aligned columns
  void* keys = take((size_t)pitch * C * (u_f32 ? 4 : 8));
  unsigned* hist = (unsigned*)take((size_t)C * kMaxTargets * kBins * sizeof(unsigned));
  Target* tg = (Target*)take((size_t)C * T * sizeof(Target));
  Target* tg_next = (Target*)take((size_t)C * T * sizeof(Target));
  double* qd = (double*)take(16 * sizeof(double));
  e = cudaMemcpyAsync(qd, q_host, nq * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  const long long tiles = ((N + 31) / 32) * ((C + 31) / 32), cap = 16LL * num_sms;
  const int gk = (int)(tiles < cap ? tiles : cap);
  if (u_f32)
    k_keys<float, uint32_t><<<gk, dim3(32, 8), 0, s>>>((const float*)u, N, C, pitch,
                                                       (uint32_t*)keys);
  else
    k_keys<double, uint64_t><<<gk, dim3(32, 8), 0, s>>>((const double*)u, N, C, pitch,
                                                        (uint64_t*)keys);
  const int gt = (C * T + 255) / 256;
  k_targets_init<<<gt, 256, 0, s>>>(C, nq, qd, N, tg);
  const size_t nh = (size_t)C * kMaxTargets * kBins;
  const int passes = u_f32 ? 4 : 8;
  // x blocks per column: enough CTAs in all to fill the GPU
  long long bx = (8LL * num_sms + C - 1) / C;
  const long long need = (N + 4 * 256 - 1) / (4 * 256);
  if (bx > need) bx = need;
  if (bx < 1) bx = 1;
  // up to kSub x 16 targets x 256 bins x 4 B = 64 KB of sub-histograms
  e = u_f32 ? cudaFuncSetAttribute(k_digit_hist<uint32_t>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, 65536)
            : cudaFuncSetAttribute(k_digit_hist<uint64_t>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, 65536);
  if (e != cudaSuccess) return e;
  for (int pass = 0; pass < passes; ++pass) {
    k_clear<<<(int)((nh + 255) / 256 < 1024 ? (nh + 255) / 256 : 1024), 256, 0, s>>>(hist, nh);
    const size_t shb = (size_t)kSub * T * kBins * sizeof(unsigned);
    if (u_f32)
      k_digit_hist<uint32_t><<<dim3((unsigned)bx, (unsigned)C), 256, shb, s>>>(
          (const uint32_t*)keys, N, pitch, C, T, pass, tg, hist);
    else
      k_digit_hist<uint64_t><<<dim3((unsigned)bx, (unsigned)C), 256, shb, s>>>(
          (const uint64_t*)keys, N, pitch, C, T, pass, tg, hist);
    k_digit_pick<<<gt, 256, 0, s>>>(C, T, pass, tg, tg_next, hist);
    std::swap(tg, tg_next);
  }
  const int gq = (C * nq + 255) / 256;
  if (u_f32) k_quantiles<uint32_t><<<gq, 256, 0, s>>>(C, nq, qd, N, tg, mscr, qv);
  else k_quantiles<uint64_t><<<gq, 256, 0, s>>>(C, nq, qd, N, tg, mscr, qv);
  return cudaGetLastError();
}

}  // namespace gbde
