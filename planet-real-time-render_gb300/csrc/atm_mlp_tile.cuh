// atm_mlp_tile.cuh - one 16-sample tile of a 64-wide MLP on the tensor cores
// (mma.sync m16n8k16, BF16 operands, FP32 accumulation).  Shared by the
// batch forward kernel and the surrogate composite.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace atm {

__host__ __device__ inline int mlp_bf16_layer_row(int in_dim) { return ((in_dim + 15) / 16) * 16 + 8; }
__host__ __device__ inline int mlp_bf16_out_pad(int out_dim) { return ((out_dim + 7) / 8) * 8; }

// Packed weights: layer l as bf16 [out_pad][in_pad + 8] (in_pad a multiple
// of 16, out_pad of 8, zero padded; the +8 bf16 row padding makes a warp's
// fragment loads conflict-free) followed by fp32 biases [out_pad].  Hidden
// layers hold W / 2 and b / 2 (see silu_half_bf16x2); the output layer W, b.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
// SiLU of two pre-activations given as halves h = z / 2 (the packed hidden
// layers are halved): z sigmoid(z) = h (1 + tanh h) = h + h tanh(h) in FP32
// (tanh.approx.f32, one MUFU op each), rounded once into the packed BF16
// pair that feeds the next layer.  (A packed tanh.approx.bf16x2 / fma.bf16x2
// form halves the MUFU work but costs the networks up to 7x their held-out
// radiance error: the activations would be rounded three times.)
__device__ __forceinline__ float silu_half(float h) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
  return fmaf(h, t, h);
}
__device__ __forceinline__ uint32_t silu_half_bf16x2(float h_lo, float h_hi) {
  return pack_bf16(silu_half(h_lo), silu_half(h_hi));
}


constexpr int kMlpH = 64;

// Runs the network on the 16 samples of a warp tile.  `x` holds each lane's
// inputs for rows g and g + 8 (k = 2q, 2q+1, 8+2q, 8+2q+1 of the first
// 16-wide chunk); returns the D fragment of the output layer (rows g, g+8,
// columns 2q, 2q+1).
template <int kMlpHidden>
__device__ __forceinline__ void mlp_tile_bf16(const unsigned char* __restrict__ w, const uint32_t (&x)[4],
                                              int in0_row, float (&y)[4]) {
  constexpr int kRow = kMlpH + 8;
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, q = lane & 3;
  uint32_t a[4][4];  // 64-wide activations as 4 k-chunks of A fragments
  // layer 0: K = 16 (inputs, zero padded), N = 64
  {
    const __nv_bfloat16* W = reinterpret_cast<const __nv_bfloat16*>(w);
    const float* b = reinterpret_cast<const float*>(w + size_t(kMlpH) * in0_row * 2);
    float c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const float b0 = b[nt * 8 + 2 * q], b1 = b[nt * 8 + 2 * q + 1];
      c[nt][0] = b0;
      c[nt][1] = b1;
      c[nt][2] = b0;
      c[nt][3] = b1;
      const __nv_bfloat16* row = W + (nt * 8 + g) * in0_row;
      mma_bf16(c[nt], x, *reinterpret_cast<const uint32_t*>(row + 2 * q),
               *reinterpret_cast<const uint32_t*>(row + 8 + 2 * q));
    }
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      a[ks][0] = silu_half_bf16x2(c[2 * ks][0], c[2 * ks][1]);
      a[ks][1] = silu_half_bf16x2(c[2 * ks][2], c[2 * ks][3]);
      a[ks][2] = silu_half_bf16x2(c[2 * ks + 1][0], c[2 * ks + 1][1]);
      a[ks][3] = silu_half_bf16x2(c[2 * ks + 1][2], c[2 * ks + 1][3]);
    }
    w += size_t(kMlpH) * in0_row * 2 + kMlpH * 4;
  }
  // hidden -> hidden layers
#pragma unroll
  for (int l = 1; l < kMlpHidden; ++l) {
    const __nv_bfloat16* W = reinterpret_cast<const __nv_bfloat16*>(w);
    const float* b = reinterpret_cast<const float*>(w + size_t(kMlpH) * kRow * 2);
    float c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const float b0 = b[nt * 8 + 2 * q], b1 = b[nt * 8 + 2 * q + 1];
      c[nt][0] = b0;
      c[nt][1] = b1;
      c[nt][2] = b0;
      c[nt][3] = b1;
      const __nv_bfloat16* row = W + (nt * 8 + g) * kRow;
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        mma_bf16(c[nt], a[ks], *reinterpret_cast<const uint32_t*>(row + ks * 16 + 2 * q),
                 *reinterpret_cast<const uint32_t*>(row + ks * 16 + 8 + 2 * q));
    }
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      a[ks][0] = silu_half_bf16x2(c[2 * ks][0], c[2 * ks][1]);
      a[ks][1] = silu_half_bf16x2(c[2 * ks][2], c[2 * ks][3]);
      a[ks][2] = silu_half_bf16x2(c[2 * ks + 1][0], c[2 * ks + 1][1]);
      a[ks][3] = silu_half_bf16x2(c[2 * ks + 1][2], c[2 * ks + 1][3]);
    }
    w += size_t(kMlpH) * kRow * 2 + kMlpH * 4;
  }
  // output layer: N = 8 (padded)
  {
    const __nv_bfloat16* W = reinterpret_cast<const __nv_bfloat16*>(w);
    const float* b = reinterpret_cast<const float*>(w + size_t(8) * kRow * 2);
    y[0] = b[2 * q];
    y[1] = b[2 * q + 1];
    y[2] = b[2 * q];
    y[3] = b[2 * q + 1];
    const __nv_bfloat16* row = W + g * kRow;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks)
      mma_bf16(y, a[ks], *reinterpret_cast<const uint32_t*>(row + ks * 16 + 2 * q),
               *reinterpret_cast<const uint32_t*>(row + ks * 16 + 8 + 2 * q));
  }
}


}  // namespace atm
