// peaks.cu -- FMA-pipe throughput microbenchmark (the roofline denominator
// for the FP64 / FP32 solver kernels).  Each thread runs 16 independent FMA
// chains so that the pipe, not the dependency latency, is the limit.
#include <cuda_runtime.h>
#include "../../include/gbde.h"

namespace gbde {

template <class T>
__global__ void __launch_bounds__(256) k_fma_peak(T* out, int iters, T a, T b) {
  T x[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = (T)(threadIdx.x + k);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = x[k] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace gbde

namespace gbde {
// Device, SM count and current stream of a context (defined in capi.cu).
int ctx_device(const gbde_ctx* ctx, int* device, int* num_sms, cudaStream_t* stream);
}  // namespace gbde

template <class T>
static int run_peak(gbde_ctx* ctx, double* tflops) {
  int dev = 0, sms = 0;
  cudaStream_t s = nullptr;
  if (gbde::ctx_device(ctx, &dev, &sms, &s) != GBDE_OK) return GBDE_ERR_INVALID;
  cudaSetDevice(dev);
  const int block = 256, grid = sms * 8;
  const int iters = sizeof(T) == 8 ? 2048 : 16384;
  T* out = nullptr;
  if (cudaMalloc(&out, (size_t)grid * block * sizeof(T)) != cudaSuccess) return GBDE_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, s);
    gbde::k_fma_peak<T><<<grid, block, 0, s>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;  // first launch is a warm-up
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return GBDE_ERR_CUDA;
  const double flops = 2.0 * 16.0 * (double)iters * grid * block;
  *tflops = flops / (best * 1e-3) / 1e12;
  return GBDE_OK;
}

extern "C" int gbde_measure_fma_peak(gbde_ctx* ctx, int32_t kind, double* tflops) {
  if (!ctx || !tflops || (kind != 0 && kind != 1)) return GBDE_ERR_INVALID;
  return kind == 0 ? run_peak<double>(ctx, tflops) : run_peak<float>(ctx, tflops);
}
