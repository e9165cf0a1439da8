// mlp.cuh -- the learned step-size / stiffness / cost predictor: a 4-layer
// MLP 8 -> 64 -> 64 -> 64 -> 3 with GELU, BF16 weights and activations as
// matrix operands, FP32 accumulation, on the tensor cores through warp-level
// mma.sync m16n8k16 (bf16 x bf16 -> f32).
//
// Inputs: 8 features of a trajectory (parameters, initial state, time span;
// models.cuh).  Outputs: y0 = normalised log10 of the first accepted step,
// y1 = logit of "Rosenbrock is cheaper than the explicit method", y2 =
// normalised log2 of the attempted steps (the trajectory's cost, which orders
// the persistent queue).
//
// Network blob (GBDE_MLP_NET_FLOATS floats, FP32 master copy):
//   W1[8][64] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64][3] b4[3]
//   x_mean[8] x_scale[8] y_mean y_scale c_mean c_scale
// Matrices are [in][out]: z = x W + b.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace gbde {
namespace mlp {

constexpr int IN = 8, HID = 64, OUT = 3;
constexpr int KIN = 16;   // IN padded to one k16 tile
constexpr int NOUT = 8;   // OUT padded to one n8 tile
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + IN * HID, OFF_W2 = OFF_B1 + HID,
              OFF_B2 = OFF_W2 + HID * HID, OFF_W3 = OFF_B2 + HID, OFF_B3 = OFF_W3 + HID * HID,
              OFF_W4 = OFF_B3 + HID, OFF_B4 = OFF_W4 + HID * OUT, NPARAM = OFF_B4 + OUT;
constexpr int OFF_XMEAN = NPARAM, OFF_XSCALE = OFF_XMEAN + IN, OFF_YMEAN = OFF_XSCALE + IN,
              OFF_YSCALE = OFF_YMEAN + 1, OFF_CMEAN = OFF_YSCALE + 1, OFF_CSCALE = OFF_CMEAN + 1,
              NET_FLOATS = OFF_CSCALE + 1;
static_assert(NPARAM == 9091 && NET_FLOATS == 9111, "parameter count");

// GELU, tanh form: 0.5 z (1 + tanh(c (z + 0.044715 z^3))), c = sqrt(2/pi)
GBDE_D float gelu(float z) {
  const float u = 0.7978845608f * (z + 0.044715f * z * z * z);
  return 0.5f * z * (1.0f + tanhf(u));
}
GBDE_D float gelu_grad(float z) {
  const float z2 = z * z;
  const float u = 0.7978845608f * (z + 0.044715f * z2 * z);
  const float th = tanhf(u);
  return 0.5f * (1.0f + th) + 0.5f * z * (1.0f - th * th) * 0.7978845608f * (1.0f + 0.134145f * z2);
}

GBDE_D uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// A strided BF16 matrix view: element (r, c) at p[r * rs + c * cs].
struct View {
  const __nv_bfloat16* p;
  int rs, cs;
  GBDE_D __nv_bfloat16 at(int r, int c) const { return p[r * rs + c * cs]; }
};

// One warp: C[16][N] (FP32, row stride ldc) = (accumulate ? C : 0) + A[16][K] B[K][N]
// with mma.sync.m16n8k16 (A row-major fragments, B column fragments).
// Fragment layout (g = lane / 4, t = lane % 4):
//   A regs: (g, 2t..2t+1) (g+8, 2t..) (g, 2t+8..) (g+8, 2t+8..)
//   B regs: (k = 2t..2t+1, n = g) (k = 2t+8.., n = g)
//   C:      (g, 2t..2t+1) (g+8, 2t..2t+1)
template <int K, int N>
GBDE_D void warp_gemm(View A, View B, float* C, int ldc, bool accumulate) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < N / 8; ++nt) {
    float c[4];
    if (accumulate) {
      c[0] = C[g * ldc + nt * 8 + 2 * t];
      c[1] = C[g * ldc + nt * 8 + 2 * t + 1];
      c[2] = C[(g + 8) * ldc + nt * 8 + 2 * t];
      c[3] = C[(g + 8) * ldc + nt * 8 + 2 * t + 1];
    } else {
      c[0] = c[1] = c[2] = c[3] = 0.0f;
    }
#pragma unroll
    for (int kt = 0; kt < K / 16; ++kt) {
      const int k0 = kt * 16 + 2 * t;
      const uint32_t a0 = pack_bf16(A.at(g, k0), A.at(g, k0 + 1));
      const uint32_t a1 = pack_bf16(A.at(g + 8, k0), A.at(g + 8, k0 + 1));
      const uint32_t a2 = pack_bf16(A.at(g, k0 + 8), A.at(g, k0 + 9));
      const uint32_t a3 = pack_bf16(A.at(g + 8, k0 + 8), A.at(g + 8, k0 + 9));
      const int n = nt * 8 + g;
      const uint32_t b0 = pack_bf16(B.at(k0, n), B.at(k0 + 1, n));
      const uint32_t b1 = pack_bf16(B.at(k0 + 8, n), B.at(k0 + 9, n));
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
          "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
          : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
    C[g * ldc + nt * 8 + 2 * t] = c[0];
    C[g * ldc + nt * 8 + 2 * t + 1] = c[1];
    C[(g + 8) * ldc + nt * 8 + 2 * t] = c[2];
    C[(g + 8) * ldc + nt * 8 + 2 * t + 1] = c[3];
  }
}

}  // namespace mlp
}  // namespace gbde
