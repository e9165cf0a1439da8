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

template <class T>
__global__ void __launch_bounds__(256) k_sum(const T* __restrict__ u, int64_t total, int C,
                                             double* __restrict__ partial) {
  // stride = gridDim.x * blockDim.x is a multiple of C: column fixed per thread
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = (int)(start % C);
  const double s = (double)u[c];
  double s1 = 0.0, s2 = 0.0;
  for (int64_t e = start; e < total; e += stride) {
    const double d = (double)u[e] - s;
    s1 += d;
    s2 += d * d;
  }
  // per-CTA column sums in fixed thread order: thread t adds into column
  // (start_t % C); threads of one column are reduced by the lowest of them
  extern __shared__ double sh[];  // [blockDim][2]
  sh[2 * threadIdx.x] = s1;
  sh[2 * threadIdx.x + 1] = s2;
  __syncthreads();
  double* out = partial + (size_t)blockIdx.x * C * 2;
  const int64_t base = (int64_t)blockIdx.x * blockDim.x;
  for (int t = threadIdx.x; t < C; t += blockDim.x) {
    // columns this CTA's threads cover: thread j has column (base + j) % C
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

template <class T>
__global__ void k_sum_final(const T* __restrict__ u, const double* __restrict__ partial,
                            int nblk, int C, int64_t N, double* __restrict__ mean,
                            double* __restrict__ var, double* __restrict__ mean_scratch) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
    double s1 = 0.0, s2 = 0.0;
    for (int b = 0; b < nblk; ++b) {
      s1 += partial[((size_t)b * C + c) * 2];
      s2 += partial[((size_t)b * C + c) * 2 + 1];
    }
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
}

template <class T, class K>
__global__ void __launch_bounds__(256) k_keys(const T* __restrict__ u, int64_t N, int C,
                                              K* __restrict__ keys) {
  // read u[i][c] row-major (coalesced), write keys[c][i]
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N * C;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / C;
    const int c = (int)(e - i * C);
    keys[(size_t)c * N + i] = ord_key(u[e]);
  }
}

// Per target (c, t): prefix of the key digits fixed so far and the rank
// still to find inside it.
struct Target {
  unsigned long long prefix;
  long long rank;
};

template <class K>
__global__ void __launch_bounds__(256) k_digit_hist(const K* __restrict__ keys, int64_t N, int C,
                                                    int T, int pass,
                                                    const Target* __restrict__ tg,
                                                    unsigned* __restrict__ hist) {
  // blockIdx.y = column; the x blocks split its N keys
  __shared__ unsigned h[kMaxTargets][kBins];
  __shared__ unsigned long long pre[kMaxTargets];
  const int c = blockIdx.y;
  constexpr int BITS = 8 * (int)sizeof(K);
  const int shift = BITS - 8 * (pass + 1);
  for (int i = threadIdx.x; i < T * kBins; i += blockDim.x) h[i / kBins][i % kBins] = 0;
  if (threadIdx.x < T) pre[threadIdx.x] = tg[(size_t)c * T + threadIdx.x].prefix;
  __syncthreads();
  const K* col = keys + (size_t)c * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const K k = col[i];
    const unsigned digit = (unsigned)((k >> shift) & 0xffu);
    if (pass == 0) {
      atomicAdd(&h[0][digit], 1u);  // every target shares the empty prefix
    } else {
      const unsigned long long hi = (unsigned long long)(k >> (shift + 8));
      for (int t = 0; t < T; ++t)
        if (hi == pre[t]) atomicAdd(&h[t][digit], 1u);
    }
  }
  __syncthreads();
  const int nt = pass == 0 ? 1 : T;
  unsigned* g = hist + (size_t)c * kMaxTargets * kBins;
  for (int i = threadIdx.x; i < nt * kBins; i += blockDim.x) {
    const unsigned v = h[i / kBins][i % kBins];
    if (v) atomicAdd(&g[i], v);
  }
}

__global__ void k_digit_pick(int C, int T, int pass, Target* __restrict__ tg,
                             unsigned* __restrict__ hist) {
  // one thread per (column, target): walk the bins to the one holding the rank
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C * T) return;
  const int c = i / T, t = i % T;
  const unsigned* h = hist + ((size_t)c * kMaxTargets + (pass == 0 ? 0 : t)) * kBins;
  Target x = tg[i];
  long long r = x.rank;
  int d = 0;
  for (; d < kBins - 1; ++d) {
    if (r < (long long)h[d]) break;
    r -= h[d];
  }
  x.prefix = (x.prefix << 8) | (unsigned long long)d;
  x.rank = r;
  tg[i] = x;
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
    b += (size_t)N * C * (u_f32 ? 4 : 8);
    b += (size_t)C * kMaxTargets * kBins * sizeof(unsigned);
    b += (size_t)C * 2 * nq * sizeof(Target);
    b += 16 * sizeof(double);
  }
  return b + 8 * 256;  // each of the (at most 6) sub-buffers is rounded up to 256 B
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
  const int g1 = (C + 255) / 256;
  if (u_f32)
    k_sum_final<float><<<g1, 256, 0, s>>>((const float*)u, partial, nblk, C, N, mean, var, mscr);
  else
    k_sum_final<double><<<g1, 256, 0, s>>>((const double*)u, partial, nblk, C, N, mean, var, mscr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nq == 0 || qv == nullptr) return e;

  const int T = 2 * nq;
  void* keys = take((size_t)N * C * (u_f32 ? 4 : 8));
  unsigned* hist = (unsigned*)take((size_t)C * kMaxTargets * kBins * sizeof(unsigned));
  Target* tg = (Target*)take((size_t)C * T * sizeof(Target));
  double* qd = (double*)take(16 * sizeof(double));
  e = cudaMemcpyAsync(qd, q_host, nq * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  const long long want = (N * C + 255) / 256, cap = 8LL * num_sms;
  const int gk = (int)(want < cap ? want : cap);
  if (u_f32) k_keys<float, uint32_t><<<gk, 256, 0, s>>>((const float*)u, N, C, (uint32_t*)keys);
  else k_keys<double, uint64_t><<<gk, 256, 0, s>>>((const double*)u, N, C, (uint64_t*)keys);
  const int gt = (C * T + 255) / 256;
  k_targets_init<<<gt, 256, 0, s>>>(C, nq, qd, N, tg);
  const size_t nh = (size_t)C * kMaxTargets * kBins;
  const int passes = u_f32 ? 4 : 8;
  // x blocks per column: enough CTAs in all to fill the GPU
  long long bx = (8LL * num_sms + C - 1) / C;
  const long long need = (N + 255) / 256;
  if (bx > need) bx = need;
  if (bx < 1) bx = 1;
  for (int pass = 0; pass < passes; ++pass) {
    k_clear<<<(int)((nh + 255) / 256 < 1024 ? (nh + 255) / 256 : 1024), 256, 0, s>>>(hist, nh);
    if (u_f32)
      k_digit_hist<uint32_t><<<dim3((unsigned)bx, (unsigned)C), 256, 0, s>>>(
          (const uint32_t*)keys, N, C, T, pass, tg, hist);
    else
      k_digit_hist<uint64_t><<<dim3((unsigned)bx, (unsigned)C), 256, 0, s>>>(
          (const uint64_t*)keys, N, C, T, pass, tg, hist);
    k_digit_pick<<<gt, 256, 0, s>>>(C, T, pass, tg, hist);
  }
  const int gq = (C * nq + 255) / 256;
  if (u_f32) k_quantiles<uint32_t><<<gq, 256, 0, s>>>(C, nq, qd, N, tg, mscr, qv);
  else k_quantiles<uint64_t><<<gq, 256, 0, s>>>(C, nq, qd, N, tg, mscr, qv);
  return cudaGetLastError();
}

}  // namespace gbde
