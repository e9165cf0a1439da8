// auto.cu -- per-trajectory method choice (GBDE_ALG_AUTO): the stand-in for
// the reference's stiffness switching (AutoTsit5(Rosenbrock23()) and friends,
// test/qa/qa.jl:15-19).  Each trajectory is classified once, before it is
// integrated -- stiff iff its stiffness parameter p[0] exceeds a threshold,
// or iff the learned predictor says so -- and the two lists run as separate
// launches of the explicit and the Rosenbrock kernel.  The adaptive error
// control of either method still judges every step.
#include <cuda_runtime.h>

#include "launch.h"

namespace gbde {

namespace {

__global__ void __launch_bounds__(256) k_partition(const double* __restrict__ p, int np,
                                                   double thr, const int8_t* __restrict__ pred,
                                                   int64_t n, unsigned* __restrict__ cnt,
                                                   int32_t* __restrict__ nonstiff,
                                                   int32_t* __restrict__ stiff) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const bool st = pred ? pred[i] != 0 : __ldg(p + (size_t)i * np) > thr;
    // warp-aggregated append to the chosen list
    const unsigned active = __activemask();
    const unsigned same = __match_any_sync(active, (int)st);
    const int leader = __ffs(same) - 1;
    const int rank = __popc(same & ((1u << (threadIdx.x & 31)) - 1));
    unsigned base = 0;
    if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(&cnt[st ? 1 : 0], __popc(same));
    base = __shfl_sync(same, base, leader);
    (st ? stiff : nonstiff)[base + rank] = (int32_t)i;
  }
}

}  // namespace

size_t partition_scratch_bytes(int64_t n) { return 2 * (size_t)n * sizeof(int32_t); }

cudaError_t build_partition(const double* p, int np, double thr, const int8_t* pred, int64_t n,
                            void* scratch, unsigned* counters, int num_sms, cudaStream_t s,
                            int32_t** nonstiff, int32_t** stiff) {
  *nonstiff = static_cast<int32_t*>(scratch);
  *stiff = *nonstiff + n;
  cudaError_t e = cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  const long long want = (n + 255) / 256;
  const int grid = (int)(want < 4LL * num_sms ? (want > 0 ? want : 1) : 4LL * num_sms);
  k_partition<<<grid, 256, 0, s>>>(p, np, thr, pred, n, counters, *nonstiff, *stiff);
  return cudaGetLastError();
}

}  // namespace gbde
