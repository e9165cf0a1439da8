// order.cu -- the order of the persistent work queue.
//
// Persistent CTAs take trajectories from the queue in this order, so the most
// expensive integrations start first and the launch does not end with a few
// long trajectories running on an otherwise idle GPU (longest-processing-
// time-first list scheduling).  Two cost keys:
//  * the span tf - t0 (no model needed): on the stiff Robertson ensemble, step
//    counts correlate with log(tf) at 0.81;
//  * the learned cost, log2 of the predicted attempted steps (mlp.cuh output
//    y2): consecutive queue positions -- the lanes of one warp -- then carry
//    trajectories of nearly equal step counts, so a warp's lanes finish
//    together instead of idling behind the longest one.
//
// A counting sort on 1024 buckets, three small kernels:
//   histogram -> exclusive scan (one CTA) -> scatter.
// Span buckets: the span's FP32 bit pattern (8 exponent bits + 2 mantissa
// bits: buckets 19% wide).  Cost buckets: log2 cost in [0, 20) in steps of
// 1/51.2 (1.4% wide).
// Order within a bucket follows atomic arrival and is not deterministic;
// each trajectory's result does not depend on it.
#include <cuda_runtime.h>

#include "launch.h"

namespace gbde {

namespace {

constexpr int kBuckets = 1024;

struct SpanKey {
  const double* t0;
  const double* tf;
  __device__ __forceinline__ int operator()(int64_t i) const {
    const float span = (float)(__ldg(tf + i) - __ldg(t0 + i));
    if (!(span > 0.0f)) return kBuckets - 1;  // empty, inverted or NaN spans last
    const unsigned key = __float_as_uint(span) >> 21;  // sign 0: key in [0, 1023]
    return kBuckets - 1 - (int)key;                    // longest first
  }
};

struct CostKey {
  const float* log2_cost;
  __device__ __forceinline__ int operator()(int64_t i) const {
    const float c = __ldg(log2_cost + i) * 51.2f;
    const int b = c > 0.0f ? (c < (float)(kBuckets - 1) ? (int)c : kBuckets - 1) : 0;  // NaN -> 0
    return kBuckets - 1 - b;  // most expensive first
  }
};

template <class Key>
__global__ void __launch_bounds__(256) k_span_hist(Key key, int64_t n, unsigned* __restrict__ hist) {
  __shared__ unsigned h[kBuckets];
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) h[b] = 0;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&h[key(i)], 1u);
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

template <class Key>
__global__ void __launch_bounds__(256) k_span_scatter(Key key, int64_t n,
                                                      unsigned* __restrict__ offs,
                                                      int32_t* __restrict__ order) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned pos = atomicAdd(&offs[key(i)], 1u);
    order[pos] = (int32_t)i;
  }
}

template <class Key>
cudaError_t build_order(Key key, int64_t n, void* scratch, int num_sms, cudaStream_t s,
                        const int32_t** order_out) {
  int32_t* order = static_cast<int32_t*>(scratch);
  unsigned* hist = reinterpret_cast<unsigned*>(order + n);
  unsigned* offs = hist + kBuckets;
  cudaError_t e = cudaMemsetAsync(hist, 0, kBuckets * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  long long want = (n + 255) / 256;
  const int grid = (int)(want < 4LL * num_sms ? (want > 0 ? want : 1) : 4LL * num_sms);
  k_span_hist<<<grid, 256, 0, s>>>(key, n, hist);
  k_span_scan<<<1, kBuckets, 0, s>>>(hist, offs);
  k_span_scatter<<<grid, 256, 0, s>>>(key, n, offs, order);
  *order_out = order;
  return cudaGetLastError();
}

}  // namespace

size_t span_order_scratch_bytes(int64_t n) {
  return (size_t)n * sizeof(int32_t) + 2 * kBuckets * sizeof(unsigned);
}

// order[0..n) = trajectory indices, longest span first.  `scratch` holds
// span_order_scratch_bytes(n) bytes (order array, then 2 x 1024 counters).
cudaError_t build_span_order(const double* t0, const double* tf, int64_t n, void* scratch,
                             int num_sms, cudaStream_t s, const int32_t** order_out) {
  return build_order(SpanKey{t0, tf}, n, scratch, num_sms, s, order_out);
}

// order[0..n) = trajectory indices, highest learned cost first; same scratch.
cudaError_t build_cost_order(const float* log2_cost, int64_t n, void* scratch, int num_sms,
                             cudaStream_t s, const int32_t** order_out) {
  return build_order(CostKey{log2_cost}, n, scratch, num_sms, s, order_out);
}

}  // namespace gbde
