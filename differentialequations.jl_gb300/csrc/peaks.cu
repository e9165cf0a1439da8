// peaks.cu -- FMA-pipe throughput microbenchmark (the roofline denominator
// for the FP64 / FP32 solver kernels).  Each thread runs 16 independent FMA
// chains so that the pipe, not the dependency latency, is the limit.
#include <cstring>
#include <cuda_runtime.h>
#include "../../include/gbde.h"
#include "controller.h"

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

// ---- self-check of rcp64 (controller.h) against the IEEE division
namespace gbde {
__global__ void __launch_bounds__(256) k_rcp64_check(int64_t n, unsigned long long* worst) {
  unsigned long long w = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    // splitmix64 of the index: mantissa in [1, 2), exponent in [-60, 60], sign
    uint64_t z = (uint64_t)i * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const double m = 1.0 + (double)(z >> 12) * 0x1p-52;
    const int e = (int)((z >> 4) % 121u) - 60;
    const double x = ldexp((z & 1) ? -m : m, e);
    const double r = rcp64(x);
    const double ref = 1.0 / x;
    const double rel = fabs(r - ref) / fabs(ref);
    const unsigned long long b = (unsigned long long)__double_as_longlong(rel);
    w = b > w ? b : w;
  }
  atomicMax(worst, w);
}
}  // namespace gbde

extern "C" int gbde_check_rcp64(gbde_ctx* ctx, int64_t n, double* max_rel_err) {
  if (!ctx || !max_rel_err || n <= 0) return GBDE_ERR_INVALID;
  int dev = 0, sms = 0;
  cudaStream_t s = nullptr;
  if (gbde::ctx_device(ctx, &dev, &sms, &s) != GBDE_OK) return GBDE_ERR_INVALID;
  cudaSetDevice(dev);
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return GBDE_ERR_NOMEM;
  unsigned long long h = 0;
  cudaMemsetAsync(d, 0, sizeof(*d), s);
  gbde::k_rcp64_check<<<sms * 4, 256, 0, s>>>(n, d);
  cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  cudaFree(d);
  if (e != cudaSuccess) return GBDE_ERR_CUDA;
  double r;
  memcpy(&r, &h, sizeof(r));
  *max_rel_err = r;
  return GBDE_OK;
}
