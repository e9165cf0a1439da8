// mlp.cu -- training and inference kernels of the learned predictor
// (mlp.cuh) and their C-ABI entry points.
//
// One CTA of 4 warps stages the BF16 weights in shared memory; each warp
// pushes 16 samples at a time through the network with mma.sync (forward),
// and for training back again (backward), accumulating the weight gradients
// of its samples in shared memory and flushing them to global memory once per
// CTA.  AdamW updates the FP32 master weights.  One training epoch (gradient
// + AdamW kernels for every minibatch) is captured once as a CUDA graph and
// replayed per epoch.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gbde.h"
#include "launch.h"
#include "mlp.cuh"

namespace gbde {
int ctx_device(const gbde_ctx* ctx, int* device, int* num_sms, cudaStream_t* stream);
int set_thread_error(int code, const char* msg);
}  // namespace gbde

using namespace gbde;
using namespace gbde::mlp;

namespace {

constexpr int WARPS = 4;
constexpr int K4 = 16;  // W4 staged as [HID][16] (cols >= OUT are zero) so dY W4^T has K = 16

struct WarpBuf {
  __nv_bfloat16 Xb[16 * KIN];  // normalised input (cols >= IN are zero)
  __nv_bfloat16 Hb[16 * HID];  // current layer input as BF16
  __nv_bfloat16 Db[16 * HID];  // dZ as BF16 (dY uses the first 16 x 16)
  float Z1[16 * HID], Z2[16 * HID], Z3[16 * HID];
  float Y[16 * NOUT];
  float D[16 * HID];    // dH / dZ (FP32)
  float Ct[16 * HID];   // one 16-row tile of a weight gradient
  float loss;
};

struct Shared {
  __nv_bfloat16 W1[KIN * HID], W2[HID * HID], W3[HID * HID], W4[HID * K4];
  float b1[HID], b2[HID], b3[HID], b4[NOUT];
  float xmean[IN], xscale[IN], ymean, yscale, cmean, cscale;
  WarpBuf w[WARPS];
};
struct SharedGrad {
  Shared s;
  float g[NPARAM + 6];  // CTA gradient accumulator
};

GBDE_D void stage_weights(Shared& S, const float* net) {
  for (int i = threadIdx.x; i < KIN * HID; i += blockDim.x) {
    const int k = i / HID, n = i % HID;
    S.W1[i] = __float2bfloat16(k < IN ? net[OFF_W1 + k * HID + n] : 0.0f);
  }
  for (int i = threadIdx.x; i < HID * HID; i += blockDim.x) {
    S.W2[i] = __float2bfloat16(net[OFF_W2 + i]);
    S.W3[i] = __float2bfloat16(net[OFF_W3 + i]);
  }
  for (int i = threadIdx.x; i < HID * K4; i += blockDim.x) {
    const int k = i / K4, n = i % K4;
    S.W4[i] = __float2bfloat16(n < OUT ? net[OFF_W4 + k * OUT + n] : 0.0f);
  }
  for (int i = threadIdx.x; i < HID; i += blockDim.x) {
    S.b1[i] = net[OFF_B1 + i];
    S.b2[i] = net[OFF_B2 + i];
    S.b3[i] = net[OFF_B3 + i];
  }
  if (threadIdx.x < NOUT) S.b4[threadIdx.x] = threadIdx.x < OUT ? net[OFF_B4 + threadIdx.x] : 0.0f;
  if (threadIdx.x < IN) {
    S.xmean[threadIdx.x] = net[OFF_XMEAN + threadIdx.x];
    S.xscale[threadIdx.x] = net[OFF_XSCALE + threadIdx.x];
  }
  if (threadIdx.x == 0) {
    S.ymean = net[OFF_YMEAN];
    S.yscale = net[OFF_YSCALE];
    S.cmean = net[OFF_CMEAN];
    S.cscale = net[OFF_CSCALE];
  }
}

// Row r of the input tile from raw features (lanes 0..15, one row each).
GBDE_D void fill_input(const Shared& S, WarpBuf& W, int lane, bool valid, const float* x) {
  if (lane < 16) {
#pragma unroll
    for (int k = 0; k < KIN; ++k) {
      float v = 0.0f;
      if (valid && k < IN) v = (x[k] - S.xmean[k]) * S.xscale[k];
      W.Xb[lane * KIN + k] = __float2bfloat16(v);
    }
  }
  __syncwarp();
}

// z = h W + b, h_next = bf16(gelu(z))
template <int K>
GBDE_D void dense_gelu(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Wt, const float* b,
                       float* Z, __nv_bfloat16* Hout) {
  warp_gemm<K, HID>(View{A, lda, 1}, View{Wt, HID, 1}, Z, HID, false);
  __syncwarp();
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < 16 * HID; i += 32) {
    const float z = Z[i] + b[i % HID];
    Z[i] = z;
    Hout[i] = __float2bfloat16(gelu(z));
  }
  __syncwarp();
}

GBDE_D void forward_tile(const Shared& S, WarpBuf& W) {
  dense_gelu<KIN>(W.Xb, KIN, S.W1, S.b1, W.Z1, W.Hb);
  dense_gelu<HID>(W.Hb, HID, S.W2, S.b2, W.Z2, W.Hb);
  dense_gelu<HID>(W.Hb, HID, S.W3, S.b3, W.Z3, W.Hb);
  warp_gemm<HID, NOUT>(View{W.Hb, HID, 1}, View{S.W4, K4, 1}, W.Y, NOUT, false);
  __syncwarp();
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < 16 * NOUT; i += 32) W.Y[i] += S.b4[i % NOUT];
  __syncwarp();
}

// h = bf16(gelu(z)) again (bit-identical to the forward pass)
GBDE_D void regelu(const float* Z, __nv_bfloat16* H) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < 16 * HID; i += 32) H[i] = __float2bfloat16(gelu(Z[i]));
  __syncwarp();
}

// dW[in][out] += A^T dZ over this tile's 16 samples; A is [16][lda] BF16
// (rows = samples), dZ BF16 in W.Db ([16][HID]); rows `in` < nin are kept.
template <int NOUTC>
GBDE_D void weight_grad(const __nv_bfloat16* A, int lda, int nin, const __nv_bfloat16* dZ,
                        int ldz, WarpBuf& W, float* g, int ld_out, int nout) {
  const int lane = threadIdx.x & 31;
  for (int mt = 0; mt * 16 < nin; ++mt) {
    warp_gemm<16, NOUTC>(View{A + mt * 16, 1, lda}, View{dZ, ldz, 1}, W.Ct, NOUTC, false);
    __syncwarp();
    for (int i = lane; i < 16 * NOUTC; i += 32) {
      const int r = mt * 16 + i / NOUTC, c = i % NOUTC;
      if (r < nin && c < nout) atomicAdd(&g[r * ld_out + c], W.Ct[i]);
    }
    __syncwarp();
  }
}

// bias gradient: column sums of D[16][n]
GBDE_D void bias_grad(const float* D, int ld, int n, float* g) {
  const int lane = threadIdx.x & 31;
  for (int c = lane; c < n; c += 32) {
    float s = 0.0f;
#pragma unroll
    for (int r = 0; r < 16; ++r) s += D[r * ld + c];
    atomicAdd(&g[c], s);
  }
}

// dZ = dH * gelu'(Z) in D (FP32) and Db (BF16)
GBDE_D void gelu_back(const float* Z, WarpBuf& W) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < 16 * HID; i += 32) {
    const float d = W.D[i] * gelu_grad(Z[i]);
    W.D[i] = d;
    W.Db[i] = __float2bfloat16(d);
  }
  __syncwarp();
}

// Loss of one tile and dY: y[0] regression on the normalised log10 of the
// first accepted step (squared error), y[1] logit of the stiff label (binary
// cross-entropy), y[2] regression on the normalised log2 of the attempted
// steps (squared error); NaN targets carry no loss.  Scaled by 1 / batch.
GBDE_D void loss_grad(const Shared& S, WarpBuf& W, int lane, bool valid, const float* tgt,
                      float inv_batch) {
  float l = 0.0f, d0 = 0.0f, d1 = 0.0f, d2 = 0.0f;
  if (lane < 16 && valid) {
    const float y0 = W.Y[lane * NOUT], y1 = W.Y[lane * NOUT + 1], y2 = W.Y[lane * NOUT + 2];
    const float t0 = tgt[0], t1 = tgt[1], t2 = tgt[2];
    if (!isnan(t0)) {
      const float tn = (t0 - S.ymean) / S.yscale;
      l += (y0 - tn) * (y0 - tn);
      d0 = 2.0f * (y0 - tn);
    }
    if (!isnan(t1)) {
      const float pr = 1.0f / (1.0f + expf(-y1));
      // log(1 + e^y) - t y, evaluated stably
      l += fmaxf(y1, 0.0f) + log1pf(expf(-fabsf(y1))) - t1 * y1;
      d1 = pr - t1;
    }
    if (!isnan(t2)) {
      const float tn = (t2 - S.cmean) / S.cscale;
      l += (y2 - tn) * (y2 - tn);
      d2 = 2.0f * (y2 - tn);
    }
  }
  if (lane < 16) {
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const float v = c == 0 ? d0 * inv_batch
                             : (c == 1 ? d1 * inv_batch : (c == 2 ? d2 * inv_batch : 0.0f));
      W.Db[lane * 16 + c] = __float2bfloat16(v);
      if (c < NOUT) W.D[lane * NOUT + c] = v;
    }
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if (lane == 0) W.loss += l * inv_batch;
  __syncwarp();
}

GBDE_D void backward_tile(const Shared& S, WarpBuf& W, float* g) {
  // layer 4: dW4 = h3^T dY, db4, dH3 = dY W4^T
  weight_grad<NOUT>(W.Hb, HID, HID, W.Db, 16, W, g + OFF_W4, OUT, OUT);
  bias_grad(W.D, NOUT, OUT, g + OFF_B4);
  __syncwarp();
  warp_gemm<16, HID>(View{W.Db, 16, 1}, View{S.W4, 1, K4}, W.D, HID, false);
  __syncwarp();
  // layer 3
  gelu_back(W.Z3, W);
  bias_grad(W.D, HID, HID, g + OFF_B3);
  regelu(W.Z2, W.Hb);
  weight_grad<HID>(W.Hb, HID, HID, W.Db, HID, W, g + OFF_W3, HID, HID);
  warp_gemm<HID, HID>(View{W.Db, HID, 1}, View{S.W3, 1, HID}, W.D, HID, false);
  __syncwarp();
  // layer 2
  gelu_back(W.Z2, W);
  bias_grad(W.D, HID, HID, g + OFF_B2);
  regelu(W.Z1, W.Hb);
  weight_grad<HID>(W.Hb, HID, HID, W.Db, HID, W, g + OFF_W2, HID, HID);
  warp_gemm<HID, HID>(View{W.Db, HID, 1}, View{S.W2, 1, HID}, W.D, HID, false);
  __syncwarp();
  // layer 1
  gelu_back(W.Z1, W);
  bias_grad(W.D, HID, HID, g + OFF_B1);
  weight_grad<HID>(W.Xb, KIN, IN, W.Db, HID, W, g + OFF_W1, HID, HID);
}

// ------------------------------------------------------------- kernels
// y[n][3] = raw network outputs (normalised log10 dt, stiff logit,
// normalised log2 steps)
__global__ void __launch_bounds__(WARPS * 32) k_mlp_forward(const float* __restrict__ net,
                                                          const float* __restrict__ x, int64_t n,
                                                          float* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Shared& S = *reinterpret_cast<Shared*>(smem_raw);
  stage_weights(S, net);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpBuf& W = S.w[warp];
  for (int64_t t0 = ((int64_t)blockIdx.x * WARPS + warp) * 16; t0 < n;
       t0 += (int64_t)gridDim.x * WARPS * 16) {
    const int64_t i = t0 + (lane & 15);
    fill_input(S, W, lane, i < n, x + (i < n ? i : 0) * IN);
    forward_tile(S, W);
    if (lane < 16 && i < n) {
#pragma unroll
      for (int c = 0; c < OUT; ++c) y[i * OUT + c] = W.Y[lane * NOUT + c];
    }
    __syncwarp();
  }
}

// grad += d(loss)/d(params) over samples perm[begin..end) (or begin..end when
// perm is NULL); loss_out += loss.  The loss is a mean over `batch`.
__global__ void __launch_bounds__(WARPS * 32) k_mlp_grad(const float* __restrict__ net,
                                                       const float* __restrict__ x,
                                                       const float* __restrict__ tgt,
                                                       const int32_t* __restrict__ perm,
                                                       int64_t begin, int64_t end, float inv_batch,
                                                       float* __restrict__ grad,
                                                       float* __restrict__ loss_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SharedGrad& SG = *reinterpret_cast<SharedGrad*>(smem_raw);
  Shared& S = SG.s;
  stage_weights(S, net);
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) SG.g[i] = 0.0f;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpBuf& W = S.w[warp];
  if (lane == 0) W.loss = 0.0f;
  __syncthreads();
  for (int64_t t0 = begin + ((int64_t)blockIdx.x * WARPS + warp) * 16; t0 < end;
       t0 += (int64_t)gridDim.x * WARPS * 16) {
    const int64_t j = t0 + (lane & 15);
    const bool valid = j < end;
    const int64_t i = valid ? (perm ? (int64_t)perm[j] : j) : 0;
    fill_input(S, W, lane, valid, x + i * IN);
    forward_tile(S, W);
    loss_grad(S, W, lane, valid, tgt + i * OUT, inv_batch);
    backward_tile(S, W, SG.g);
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x)
    if (SG.g[i] != 0.0f) atomicAdd(&grad[i], SG.g[i]);
  if (lane == 0) atomicAdd(loss_out, W.loss);
}

// AdamW on the FP32 master weights (decoupled weight decay on matrices only).
// step[0] counts completed updates (advanced by k_step after this kernel).
__global__ void k_adamw(float* __restrict__ net, const float* __restrict__ grad,
                        float* __restrict__ m, float* __restrict__ v, const unsigned* step,
                        float lr, float wd, float b1, float b2, float eps) {
  const unsigned t = *step + 1;
  const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x) {
    const float gi = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const bool is_bias = (i >= OFF_B1 && i < OFF_W2) || (i >= OFF_B2 && i < OFF_W3) ||
                         (i >= OFF_B3 && i < OFF_W4) || i >= OFF_B4;
    const float upd = (mi / c1) / (sqrtf(vi / c2) + eps) + (is_bias ? 0.0f : wd * net[i]);
    net[i] -= lr * upd;
  }
}

__global__ void k_step(unsigned* step) { *step += 1; }

// Learned predictions for a solve: features -> network -> first dt, stiff
// label and log2 of the attempted steps per trajectory.  A forward-only
// kernel with the activations in registers: the m16n8 accumulators of one
// layer, after bias and GELU, are packed to BF16 pairs that are exactly the
// A fragments of the next layer's k16 tiles (n-tiles 2k, 2k+1 -> k-tile k).
// The weights sit transposed in shared memory ([out][in]) so every B
// fragment is one 32-bit load; each warp runs 16 trajectories.
struct PredShared {
  __nv_bfloat16 W1t[HID * KIN], W2t[HID * HID], W3t[HID * HID], W4t[NOUT * HID];
  float b1[HID], b2[HID], b3[HID], b4[NOUT];
  float xmean[IN], xscale[IN], ymean, yscale, cmean, cscale;
};

GBDE_D uint32_t ld_pair(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

GBDE_D uint32_t pack_f2(float lo, float hi) {
  return pack_bf16(__float2bfloat16(lo), __float2bfloat16(hi));
}

GBDE_D void mma16816(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                     uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// One hidden layer (K inputs as KT k-tiles of A fragments, 64 outputs):
// h_out[nt][0..1] = BF16 pairs of gelu(A W + b) for rows g and g + 8.
template <int KT>
GBDE_D void pred_layer(const uint32_t (*A)[4], const __nv_bfloat16* Wt, int ldw, const float* b,
                       uint32_t (*H)[2], int g, int t) {
#pragma unroll
  for (int nt = 0; nt < HID / 8; ++nt) {
    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const __nv_bfloat16* w = Wt + (nt * 8 + g) * ldw + 2 * t;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
      mma16816(c, A[kt][0], A[kt][1], A[kt][2], A[kt][3], ld_pair(w + kt * 16),
               ld_pair(w + kt * 16 + 8));
    const float b0 = b[nt * 8 + 2 * t], b1 = b[nt * 8 + 2 * t + 1];
    H[nt][0] = pack_f2(gelu(c[0] + b0), gelu(c[1] + b1));  // row g
    H[nt][1] = pack_f2(gelu(c[2] + b0), gelu(c[3] + b1));  // row g + 8
  }
}

template <class M>
__global__ void __launch_bounds__(256) k_mlp_predict(const float* __restrict__ net,
                                                     const double* __restrict__ p,
                                                     const double* __restrict__ u0,
                                                     const double* __restrict__ t0,
                                                     const double* __restrict__ tf, int64_t n,
                                                     float* __restrict__ pred_dt,
                                                     int8_t* __restrict__ pred_stiff,
                                                     float* __restrict__ pred_cost) {
  __shared__ PredShared S;
  for (int i = threadIdx.x; i < HID * KIN; i += blockDim.x) {
    const int o = i / KIN, k = i % KIN;
    S.W1t[i] = __float2bfloat16(k < IN ? net[OFF_W1 + k * HID + o] : 0.0f);
  }
  for (int i = threadIdx.x; i < HID * HID; i += blockDim.x) {
    const int o = i / HID, k = i % HID;
    S.W2t[i] = __float2bfloat16(net[OFF_W2 + k * HID + o]);
    S.W3t[i] = __float2bfloat16(net[OFF_W3 + k * HID + o]);
  }
  for (int i = threadIdx.x; i < NOUT * HID; i += blockDim.x) {
    const int o = i / HID, k = i % HID;
    S.W4t[i] = __float2bfloat16(o < OUT ? net[OFF_W4 + k * OUT + o] : 0.0f);
  }
  for (int i = threadIdx.x; i < HID; i += blockDim.x) {
    S.b1[i] = net[OFF_B1 + i];
    S.b2[i] = net[OFF_B2 + i];
    S.b3[i] = net[OFF_B3 + i];
  }
  if (threadIdx.x < NOUT) S.b4[threadIdx.x] = threadIdx.x < OUT ? net[OFF_B4 + threadIdx.x] : 0.0f;
  if (threadIdx.x < IN) {
    S.xmean[threadIdx.x] = net[OFF_XMEAN + threadIdx.x];
    S.xscale[threadIdx.x] = net[OFF_XSCALE + threadIdx.x];
  }
  if (threadIdx.x == 0) {
    S.ymean = net[OFF_YMEAN];
    S.yscale = net[OFF_YSCALE];
    S.cmean = net[OFF_CMEAN];
    S.cscale = net[OFF_CSCALE];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b0 = wid * 16; b0 < n; b0 += nw * 16) {
    // lanes 0..15: normalised features of trajectory b0 + lane
    float x[IN];
    {
      const int64_t i = b0 + (lane & 15);
      float f[IN];
#pragma unroll
      for (int k = 0; k < IN; ++k) f[k] = 0.0f;
      if (lane < 16 && i < n) M::features(p + i * M::NP, u0 + i * M::N, tf[i] - t0[i], f);
#pragma unroll
      for (int k = 0; k < IN; ++k) x[k] = lane < 16 && i < n ? (f[k] - S.xmean[k]) * S.xscale[k] : 0.0f;
    }
    // layer 1 A fragment (K = 16, inputs 8..15 zero): rows g and g + 8, k = 2t, 2t + 1
    uint32_t A1[1][4];
    {
      float r0[2], r1[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        float v0 = 0.0f, v1 = 0.0f;
#pragma unroll
        for (int k = 0; k < IN; ++k) {
          const float a = __shfl_sync(0xffffffffu, x[k], g);
          const float bq = __shfl_sync(0xffffffffu, x[k], g + 8);
          if (k == 2 * t + q) {
            v0 = a;
            v1 = bq;
          }
        }
        r0[q] = v0;
        r1[q] = v1;
      }
      A1[0][0] = pack_f2(r0[0], r0[1]);
      A1[0][1] = pack_f2(r1[0], r1[1]);
      A1[0][2] = 0u;
      A1[0][3] = 0u;
    }
    uint32_t H[HID / 8][2], A[HID / 16][4];
    pred_layer<1>(A1, S.W1t, KIN, S.b1, H, g, t);
#pragma unroll
    for (int kt = 0; kt < HID / 16; ++kt) {
      A[kt][0] = H[2 * kt][0];
      A[kt][1] = H[2 * kt][1];
      A[kt][2] = H[2 * kt + 1][0];
      A[kt][3] = H[2 * kt + 1][1];
    }
    pred_layer<HID / 16>(A, S.W2t, HID, S.b2, H, g, t);
#pragma unroll
    for (int kt = 0; kt < HID / 16; ++kt) {
      A[kt][0] = H[2 * kt][0];
      A[kt][1] = H[2 * kt][1];
      A[kt][2] = H[2 * kt + 1][0];
      A[kt][3] = H[2 * kt + 1][1];
    }
    pred_layer<HID / 16>(A, S.W3t, HID, S.b3, H, g, t);
    // output layer: one n8 tile; lane (g, t) holds outputs 2t, 2t + 1 of rows g, g + 8
    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const __nv_bfloat16* w = S.W4t + g * HID + 2 * t;
#pragma unroll
    for (int kt = 0; kt < HID / 16; ++kt)
      mma16816(c, H[2 * kt][0], H[2 * kt][1], H[2 * kt + 1][0], H[2 * kt + 1][1],
               ld_pair(w + kt * 16), ld_pair(w + kt * 16 + 8));
    const float o0 = S.b4[2 * t], o1 = S.b4[2 * t + 1];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int64_t i = b0 + g + 8 * r;
      const float ya = c[2 * r] + o0, yb = c[2 * r + 1] + o1;
      if (i < n) {
        if (t == 0) {
          const float l10 = ya * S.yscale + S.ymean;
          pred_dt[i] = exp10f(fminf(fmaxf(l10, -30.0f), 30.0f));
          pred_stiff[i] = yb > 0.0f ? 1 : 0;
        } else if (t == 1) {
          pred_cost[i] = ya * S.cscale + S.cmean;
        }
      }
    }
  }
}

template <class M>
__global__ void k_features(const double* __restrict__ p, const double* __restrict__ u0,
                           const double* __restrict__ t0, const double* __restrict__ tf,
                           int64_t n, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    M::features(p + i * M::NP, u0 + i * M::N, tf[i] - t0[i], out + i * IN);
}

int fail(int code, const char* msg) { return set_thread_error(code, msg); }

#define MLP_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      char b_[256];                                                                     \
      snprintf(b_, sizeof(b_), "%s failed: %s", #call, cudaGetErrorString(e_));         \
      return fail(e_ == cudaErrorMemoryAllocation ? GBDE_ERR_NOMEM : GBDE_ERR_CUDA, b_); \
    }                                                                                   \
  } while (0)

// RAII device buffers for the MLP entry points (transient, per call).
struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t b) { return cudaMalloc(&p, b < 16 ? 16 : b); }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

template <class K>
cudaError_t set_smem(K kern, size_t bytes) {
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int grid_for(int64_t n, int num_sms) {
  const int64_t tiles = (n + WARPS * 16 - 1) / (WARPS * 16);
  const int64_t g = tiles < 2LL * num_sms ? tiles : 2LL * num_sms;
  return (int)(g > 0 ? g : 1);
}

}  // namespace

namespace gbde {
// Launch the learned predictions for model `model` (used by capi.cu).
cudaError_t mlp_predict(int model, const float* net, const KArgs& a, float* pred_dt,
                        int8_t* pred_stiff, float* pred_cost, int num_sms, cudaStream_t s) {
  // 8 warps of 16 trajectories per CTA, one wave where possible
  const long long want = (a.N + 127) / 128, cap = 8LL * num_sms;
  const int grid = (int)(want < cap ? (want > 0 ? want : 1) : cap);
  switch (model) {
#define GBDE_PRED(ID, M)                                                                  \
  case ID: {                                                                              \
    k_mlp_predict<M><<<grid, 256, 0, s>>>(net, a.p, a.u0, a.t0, a.tf,                     \
                                                               a.N, pred_dt, pred_stiff,  \
                                                               pred_cost);                \
    return cudaGetLastError();                                                            \
  }
    GBDE_PRED(GBDE_MODEL_LINEAR, Linear)
    GBDE_PRED(GBDE_MODEL_LORENZ, Lorenz)
    GBDE_PRED(GBDE_MODEL_ROBERTSON, Robertson)
    GBDE_PRED(GBDE_MODEL_VDP_RING8, VdpRing8)
    GBDE_PRED(GBDE_MODEL_LOTKA_VOLTERRA, LotkaVolterra)
#undef GBDE_PRED
  }
  return cudaErrorNotSupported;
}
}  // namespace gbde

extern "C" {

int gbde_mlp_init(uint64_t seed, float* net) {
  if (!net) return fail(GBDE_ERR_INVALID, "net is NULL");
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<float> u(-1.0f, 1.0f);
  auto fill = [&](int off, int fan_in, int count) {
    const float a = std::sqrt(6.0f / (float)fan_in);  // He-uniform for GELU layers
    for (int i = 0; i < count; ++i) net[off + i] = a * u(rng);
  };
  std::memset(net, 0, sizeof(float) * NET_FLOATS);
  fill(OFF_W1, IN, IN * HID);
  fill(OFF_W2, HID, HID * HID);
  fill(OFF_W3, HID, HID * HID);
  fill(OFF_W4, HID, HID * OUT);
  for (int k = 0; k < IN; ++k) net[OFF_XSCALE + k] = 1.0f;
  net[OFF_YSCALE] = 1.0f;
  net[OFF_CSCALE] = 1.0f;
  return GBDE_OK;
}

int gbde_mlp_features(gbde_ctx* ctx, const gbde_problem* prob, float* out) {
  if (!ctx || !prob || !out) return fail(GBDE_ERR_INVALID, "NULL argument");
  if (prob->mem != GBDE_MEM_DEVICE)
    return fail(GBDE_ERR_INVALID, "gbde_mlp_features takes device pointers (GBDE_MEM_DEVICE)");
  int dev = 0, sms = 0;
  cudaStream_t s = nullptr;
  ctx_device(ctx, &dev, &sms, &s);
  MLP_CUDA(cudaSetDevice(dev));
  const int64_t n = prob->n_traj;
  if (n <= 0) return GBDE_OK;
  const int grid = (int)((n + 255) / 256 < 4LL * sms ? (n + 255) / 256 : 4LL * sms);
  switch (prob->model) {
#define GBDE_FEAT(ID, M)                                                                    \
  case ID:                                                                                  \
    k_features<M><<<grid, 256, 0, s>>>(prob->p, prob->u0, prob->t0, prob->tf, n, out);      \
    break;
    GBDE_FEAT(GBDE_MODEL_LINEAR, Linear)
    GBDE_FEAT(GBDE_MODEL_LORENZ, Lorenz)
    GBDE_FEAT(GBDE_MODEL_ROBERTSON, Robertson)
    GBDE_FEAT(GBDE_MODEL_VDP_RING8, VdpRing8)
    GBDE_FEAT(GBDE_MODEL_LOTKA_VOLTERRA, LotkaVolterra)
#undef GBDE_FEAT
    default:
      return fail(GBDE_ERR_INVALID, "unknown model id");
  }
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaStreamSynchronize(s));
  return GBDE_OK;
}

int gbde_mlp_forward(gbde_ctx* ctx, const float* net, const float* x, int64_t n, float* y) {
  if (!ctx || !net || (n > 0 && (!x || !y))) return fail(GBDE_ERR_INVALID, "NULL argument");
  if (n <= 0) return GBDE_OK;
  int dev = 0, sms = 0;
  cudaStream_t s = nullptr;
  ctx_device(ctx, &dev, &sms, &s);
  MLP_CUDA(cudaSetDevice(dev));
  Dev dnet, dx, dy;
  MLP_CUDA(dnet.alloc(sizeof(float) * NET_FLOATS));
  MLP_CUDA(dx.alloc(sizeof(float) * IN * n));
  MLP_CUDA(dy.alloc(sizeof(float) * OUT * n));
  MLP_CUDA(cudaMemcpyAsync(dnet.p, net, sizeof(float) * NET_FLOATS, cudaMemcpyHostToDevice, s));
  MLP_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * IN * n, cudaMemcpyHostToDevice, s));
  MLP_CUDA(set_smem(k_mlp_forward, sizeof(Shared)));
  k_mlp_forward<<<grid_for(n, sms), WARPS * 32, sizeof(Shared), s>>>(dnet.as<float>(),
                                                                      dx.as<float>(), n,
                                                                      dy.as<float>());
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemcpyAsync(y, dy.p, sizeof(float) * OUT * n, cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaStreamSynchronize(s));
  return GBDE_OK;
}

int gbde_mlp_grad(gbde_ctx* ctx, const float* net, const float* x, const float* y, int64_t n,
                  float* grad, float* loss) {
  if (!ctx || !net || !grad || !loss || (n > 0 && (!x || !y)))
    return fail(GBDE_ERR_INVALID, "NULL argument");
  if (n <= 0) return fail(GBDE_ERR_INVALID, "n must be > 0");
  int dev = 0, sms = 0;
  cudaStream_t s = nullptr;
  ctx_device(ctx, &dev, &sms, &s);
  MLP_CUDA(cudaSetDevice(dev));
  Dev dnet, dx, dy, dg;
  MLP_CUDA(dnet.alloc(sizeof(float) * NET_FLOATS));
  MLP_CUDA(dx.alloc(sizeof(float) * IN * n));
  MLP_CUDA(dy.alloc(sizeof(float) * OUT * n));
  MLP_CUDA(dg.alloc(sizeof(float) * (NPARAM + 1)));
  MLP_CUDA(cudaMemcpyAsync(dnet.p, net, sizeof(float) * NET_FLOATS, cudaMemcpyHostToDevice, s));
  MLP_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * IN * n, cudaMemcpyHostToDevice, s));
  MLP_CUDA(cudaMemcpyAsync(dy.p, y, sizeof(float) * OUT * n, cudaMemcpyHostToDevice, s));
  MLP_CUDA(cudaMemsetAsync(dg.p, 0, sizeof(float) * (NPARAM + 1), s));
  MLP_CUDA(set_smem(k_mlp_grad, sizeof(SharedGrad)));
  k_mlp_grad<<<grid_for(n, sms), WARPS * 32, sizeof(SharedGrad), s>>>(
      dnet.as<float>(), dx.as<float>(), dy.as<float>(), nullptr, 0, n, 1.0f / (float)n,
      dg.as<float>(), dg.as<float>() + NPARAM);
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemcpyAsync(grad, dg.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaMemcpyAsync(loss, dg.as<float>() + NPARAM, sizeof(float), cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaStreamSynchronize(s));
  return GBDE_OK;
}

int gbde_mlp_train(gbde_ctx* ctx, const float* x, const float* y, int64_t n,
                   const gbde_mlp_train_opts* o, float* net, float* loss_history) {
  if (!ctx || !x || !y || !o || !net) return fail(GBDE_ERR_INVALID, "NULL argument");
  if (n <= 0 || o->epochs <= 0 || o->batch <= 0 || !(o->lr > 0.0f))
    return fail(GBDE_ERR_INVALID, "need n > 0, epochs > 0, batch > 0, lr > 0");
  if (n > INT32_MAX) return fail(GBDE_ERR_INVALID, "n must be < 2^31");
  int dev = 0, sms = 0;
  cudaStream_t s = nullptr;
  ctx_device(ctx, &dev, &sms, &s);
  MLP_CUDA(cudaSetDevice(dev));
  // normalisation from the data: features to zero mean / unit scale, the
  // log10-dt and log2-steps targets likewise
  std::vector<double> mean(IN, 0.0), sq(IN, 0.0);
  double ym[2] = {0.0, 0.0}, ysq[2] = {0.0, 0.0};
  int64_t ny[2] = {0, 0};
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < IN; ++k) {
      mean[k] += x[i * IN + k];
      sq[k] += (double)x[i * IN + k] * x[i * IN + k];
    }
    for (int r = 0; r < 2; ++r) {
      const float v = y[i * OUT + (r == 0 ? 0 : 2)];
      if (!std::isnan(v)) {
        ym[r] += v;
        ysq[r] += (double)v * v;
        ++ny[r];
      }
    }
  }
  for (int k = 0; k < IN; ++k) {
    const double m = mean[k] / n, var = sq[k] / n - m * m;
    net[OFF_XMEAN + k] = (float)m;
    net[OFF_XSCALE + k] = (float)(1.0 / std::sqrt(var > 1e-12 ? var : 1e-12));
  }
  for (int r = 0; r < 2; ++r) {
    if (ny[r] == 0) continue;
    const double m = ym[r] / ny[r], var = ysq[r] / ny[r] - m * m;
    net[r == 0 ? OFF_YMEAN : OFF_CMEAN] = (float)m;
    net[r == 0 ? OFF_YSCALE : OFF_CSCALE] = (float)std::sqrt(var > 1e-12 ? var : 1e-12);
  }
  Dev dnet, dx, dy, dg, dm, dv, dperm, dstep, dloss;
  MLP_CUDA(dnet.alloc(sizeof(float) * NET_FLOATS));
  MLP_CUDA(dx.alloc(sizeof(float) * IN * n));
  MLP_CUDA(dy.alloc(sizeof(float) * OUT * n));
  MLP_CUDA(dg.alloc(sizeof(float) * NPARAM));
  MLP_CUDA(dm.alloc(sizeof(float) * NPARAM));
  MLP_CUDA(dv.alloc(sizeof(float) * NPARAM));
  MLP_CUDA(dperm.alloc(sizeof(int32_t) * n));
  MLP_CUDA(dstep.alloc(sizeof(unsigned)));
  MLP_CUDA(dloss.alloc(sizeof(float)));
  MLP_CUDA(cudaMemcpyAsync(dnet.p, net, sizeof(float) * NET_FLOATS, cudaMemcpyHostToDevice, s));
  MLP_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * IN * n, cudaMemcpyHostToDevice, s));
  MLP_CUDA(cudaMemcpyAsync(dy.p, y, sizeof(float) * OUT * n, cudaMemcpyHostToDevice, s));
  MLP_CUDA(cudaMemsetAsync(dm.p, 0, sizeof(float) * NPARAM, s));
  MLP_CUDA(cudaMemsetAsync(dv.p, 0, sizeof(float) * NPARAM, s));
  MLP_CUDA(cudaMemsetAsync(dstep.p, 0, sizeof(unsigned), s));
  MLP_CUDA(set_smem(k_mlp_grad, sizeof(SharedGrad)));
  const int64_t B = o->batch < n ? o->batch : n;
  const int64_t nb = n / B;  // full minibatches per epoch
  std::vector<int32_t> perm(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = (int32_t)i;
  std::mt19937_64 rng(o->seed);
  // capture one epoch (every minibatch's gradient + AdamW) as a CUDA graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  MLP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaError_t ce = cudaMemsetAsync(dloss.p, 0, sizeof(float), s);
  for (int64_t b = 0; b < nb && ce == cudaSuccess; ++b) {
    ce = cudaMemsetAsync(dg.p, 0, sizeof(float) * NPARAM, s);
    if (ce != cudaSuccess) break;
    k_mlp_grad<<<grid_for(B, sms), WARPS * 32, sizeof(SharedGrad), s>>>(
        dnet.as<float>(), dx.as<float>(), dy.as<float>(), dperm.as<int32_t>(), b * B,
        (b + 1) * B, 1.0f / (float)B, dg.as<float>(), dloss.as<float>());
    k_adamw<<<(NPARAM + 255) / 256, 256, 0, s>>>(dnet.as<float>(), dg.as<float>(),
                                                 dm.as<float>(), dv.as<float>(),
                                                 dstep.as<unsigned>(), o->lr, o->weight_decay,
                                                 0.9f, 0.999f, 1e-8f);
    k_step<<<1, 1, 0, s>>>(dstep.as<unsigned>());
    ce = cudaGetLastError();
  }
  const cudaError_t ee = cudaStreamEndCapture(s, &graph);
  if (ce != cudaSuccess || ee != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail(GBDE_ERR_CUDA, "capturing the training epoch failed");
  }
  ce = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return fail(GBDE_ERR_CUDA, "cudaGraphInstantiate failed");
  int rc = GBDE_OK;
  for (int ep = 0; ep < o->epochs && rc == GBDE_OK; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    cudaError_t e = cudaMemcpyAsync(dperm.p, perm.data(), sizeof(int32_t) * n,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
    float l = 0.0f;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&l, dloss.p, sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = fail(GBDE_ERR_CUDA, cudaGetErrorString(e));
    else if (loss_history) loss_history[ep] = l / (float)nb;
  }
  cudaGraphExecDestroy(exec);
  if (rc != GBDE_OK) return rc;
  MLP_CUDA(cudaMemcpyAsync(net, dnet.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaStreamSynchronize(s));
  return GBDE_OK;
}

}  // extern "C"
