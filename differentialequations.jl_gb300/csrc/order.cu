// order.cu -- longest-span-first order of the persistent work queue.
//
// Persistent CTAs take trajectories from the queue in this order, so the
// longest integrations start first and the launch does not end with a few
// long trajectories running on an otherwise idle GPU (longest-processing-
// time-first list scheduling).  The span tf - t0 is the cost proxy: on the
// stiff Robertson ensemble, step counts correlate with log(tf) at 0.81.
//
// A counting sort on 1024 buckets of the span's FP32 bit pattern (8 exponent
// bits + 2 mantissa bits: buckets 19% wide), three small kernels:
//   histogram -> exclusive scan (one CTA) -> scatter.
// Order within a bucket follows atomic arrival and is not deterministic;
// each trajectory's result does not depend on it.
#include <cuda_runtime.h>

#include "launch.h"

namespace gbde {

namespace {

constexpr int kBuckets = 1024;

__device__ __forceinline__ int span_bucket(double t0, double tf) {
  const float span = (float)(tf - t0);
  if (!(span > 0.0f)) return kBuckets - 1;  // empty, inverted or NaN spans last
  const unsigned key = __float_as_uint(span) >> 21;  // sign 0: key in [0, 1023]
  return kBuckets - 1 - (int)key;                    // longest first
}

__global__ void __launch_bounds__(256) k_span_hist(const double* __restrict__ t0,
                                                   const double* __restrict__ tf, int64_t n,
                                                   unsigned* __restrict__ hist) {
  __shared__ unsigned h[kBuckets];
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) h[b] = 0;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&h[span_bucket(__ldg(t0 + i), __ldg(tf + i))], 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
}

// Exclusive scan of kBuckets counts with one CTA of kBuckets threads.
__global__ void __launch_bounds__(kBuckets) k_span_scan(const unsigned* __restrict__ hist,
                                                        unsigned* __restrict__ offs) {
  __shared__ unsigned s[kBuckets];
  const int t = threadIdx.x;
  const unsigned v = hist[t];
  s[t] = v;
  __syncthreads();
  for (int d = 1; d < kBuckets; d <<= 1) {
    const unsigned x = t >= d ? s[t - d] : 0u;
    __syncthreads();
    s[t] += x;
    __syncthreads();
  }
  offs[t] = s[t] - v;
}

__global__ void __launch_bounds__(256) k_span_scatter(const double* __restrict__ t0,
                                                      const double* __restrict__ tf, int64_t n,
                                                      unsigned* __restrict__ offs,
                                                      int32_t* __restrict__ order) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned pos = atomicAdd(&offs[span_bucket(__ldg(t0 + i), __ldg(tf + i))], 1u);
    order[pos] = (int32_t)i;
  }
}

}  // namespace

size_t span_order_scratch_bytes(int64_t n) {
  return (size_t)n * sizeof(int32_t) + 2 * kBuckets * sizeof(unsigned);
}

// order[0..n) = trajectory indices, longest span first.  `scratch` holds
// span_order_scratch_bytes(n) bytes (order array, then 2 x 1024 counters).
cudaError_t build_span_order(const double* t0, const double* tf, int64_t n, void* scratch,
                             int num_sms, cudaStream_t s, const int32_t** order_out) {
  int32_t* order = static_cast<int32_t*>(scratch);
  unsigned* hist = reinterpret_cast<unsigned*>(order + n);
  unsigned* offs = hist + kBuckets;
  cudaError_t e = cudaMemsetAsync(hist, 0, kBuckets * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  long long want = (n + 255) / 256;
  const int grid = (int)(want < 4LL * num_sms ? (want > 0 ? want : 1) : 4LL * num_sms);
  k_span_hist<<<grid, 256, 0, s>>>(t0, tf, n, hist);
  k_span_scan<<<1, kBuckets, 0, s>>>(hist, offs);
  k_span_scatter<<<grid, 256, 0, s>>>(t0, tf, n, offs, order);
  *order_out = order;
  return cudaGetLastError();
}

}  // namespace gbde
