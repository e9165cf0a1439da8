// peaks.cu -- throughput microbenchmarks, the roofline denominators of the
// solver kernels: the FP64 / FP32 FMA pipes (each thread runs 16 independent
// FMA chains, so that the pipe, not the dependency latency, is the limit) and
// the rate of the SDE kernels' normal stream (Philox4x32-10 on the integer
// pipe, Box-Muller on the MUFU pipe), generated exactly as the kernels do.
#include <cstring>
#include <cuda_runtime.h>
#include "../../include/gbde.h"
#include "controller.h"
#include "philox.h"

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

// Each thread draws `iters` blocks of four FP32 normals from its own stream
// (the layout of NormalStream<float> in sde.cuh) and keeps their sum.
__global__ void __launch_bounds__(256) k_normal_peak(float* out, int iters, uint64_t seed) {
  const uint64_t tr = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.0f;
  for (int b = 0; b < iters; ++b) {
    float z[4];
    philox_normal_quad_f32(seed, tr, (uint64_t)b, z);
    acc += (z[0] + z[1]) + (z[2] + z[3]);
  }
  out[tr] = acc;
}

}  // namespace gbde

namespace gbde {
// Device, SM count and current stream of a context (defined in capi.cu).
int ctx_device(const gbde_ctx* ctx, int* device, int* num_sms, cudaStream_t* stream);
}  // namespace gbde

// kind: 0 = FP64 FMA, 1 = FP32 FMA (T the FMA type), 2 = FP32 normals (T = float)
template <class T>
static int run_peak(gbde_ctx* ctx, double* tflops, int kind) {
  int dev = 0, sms = 0;
  cudaStream_t s = nullptr;
  if (gbde::ctx_device(ctx, &dev, &sms, &s) != GBDE_OK) return GBDE_ERR_INVALID;
  cudaSetDevice(dev);
  const int block = 256, grid = sms * 8;
  const int iters = kind == 2 ? 256 : (sizeof(T) == 8 ? 2048 : 16384);
  T* out = nullptr;
  if (cudaMalloc(&out, (size_t)grid * block * sizeof(T)) != cudaSuccess) return GBDE_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, s);
    if (kind == 2)
      gbde::k_normal_peak<<<grid, block, 0, s>>>((float*)out, iters, 20261204ull + rep);
    else
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
  // FMA = 2 flops; a normal counts as one unit
  const double work = (kind == 2 ? 4.0 : 2.0 * 16.0) * (double)iters * grid * block;
  *tflops = work / (best * 1e-3) / 1e12;
  return GBDE_OK;
}

extern "C" int gbde_measure_fma_peak(gbde_ctx* ctx, int32_t kind, double* tflops) {
  if (!ctx || !tflops || kind < 0 || kind > 2) return GBDE_ERR_INVALID;
  if (kind == 0) return run_peak<double>(ctx, tflops, 0);
  return run_peak<float>(ctx, tflops, kind);
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
