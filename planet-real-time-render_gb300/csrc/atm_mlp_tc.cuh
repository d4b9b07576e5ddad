// atm_mlp_tc.cuh - a 64-wide SiLU MLP on 128-row tiles with tcgen05.mma:
// activations in tensor memory (the A operand), weights in shared memory
// (the B operand, read by the tensor core through descriptors), FP32
// accumulators in tensor memory, SiLU epilogue per row by the thread that
// owns the row.  Shared by the batch forward kernel and the surrogate
// composite.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "atm_kernels.h"
#include "atm_mlp_tile.cuh"
#include "atm_tc.cuh"

namespace atm {

// Packed tcgen05 layout of one network: per layer the weights as K-major core
// matrices (atm_tc.cuh), K padded to 16 (first layer) or 64, N to 64
// (hidden) or 16 (output; the M = 128 MMA takes N in steps of 16), then the
// FP32 biases [N_pad].  Hidden layers hold W / 2 and b / 2 (SiLU of halves).
__host__ __device__ inline int tc_k_pad(int in_dim) { return ((in_dim + 15) / 16) * 16; }
__host__ __device__ inline int tc_n_pad(int out_dim) { return ((out_dim + 15) / 16) * 16; }
__host__ __device__ inline int tc_layer_bytes(int in_dim, int out_dim) {
  return tc_k_pad(in_dim) * tc_n_pad(out_dim) * 2 + tc_n_pad(out_dim) * 4;
}
// Byte offset of element (n, k) inside a layer's weight block.
__host__ __device__ inline int tc_w_offset(int n, int k, int n_pad) {
  const int s = k >> 4, i = (k >> 3) & 1, j = n >> 3, r = n & 7, e = k & 7;
  return (((s * (n_pad >> 3) + j) * 2 + i) << 7) + r * 16 + e * 2;
}

constexpr uint32_t kTcLbo = 128;  // K-adjacent core matrices
constexpr uint32_t kTcSbo = 256;  // N-adjacent core matrices

// Per-tile state of a network run.
struct TcTile {
  uint32_t tmem_d;   // accumulator columns (64), lane 0
  uint32_t tmem_a;   // activation columns (32), lane 0
  uint64_t* mbar;    // MMA completion
  uint32_t phase;    // parity of the next completion
  int tile;          // index of the tile in the CTA (named barrier 1 + tile)
  int row;           // this thread's row 0..127
};

// Runs the network (n_in <= 16 inputs, kHidden layers of 64, n_out <= 8) for
// the tile's 128 rows; every thread of the tile calls with its row's inputs
// (unused ones zero) and receives its row's outputs.  w: generic pointer to the packed network
// in shared memory.  Each completion wait polls the mbarrier at most
// wait_tries times.  Returns false, in every thread of the tile, if a layer's
// MMAs did not complete in time: the outputs are then not valid, no further
// MMA was issued, and exactly one commit (parity T.phase ^ 1) may still be
// in flight - the caller waits for it before it frees the tensor memory.
template <int kHidden>
__device__ __forceinline__ bool mlp_tile_tc(const unsigned char* w, int n_in, TcTile& T, const float (&x)[16],
                                            float (&y)[8], int wait_tries = kTcWaitTries) {
  const uint32_t lane_off = uint32_t(T.row & ~31) << 16;  // the warp's quarter of the lanes
  const bool issuer = T.row == 0;
  // inputs -> A columns 0..7 (K = 16, BF16 pairs)
  {
    uint32_t v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = pack_bf16(x[2 * i], x[2 * i + 1]);
    tc::st8(T.tmem_a + lane_off, v);
    tc::wait_st();
  }
  const uint32_t w_saddr = tc::smem_addr(w);
  int off = 0;
  int in_dim = n_in;
#pragma unroll
  for (int l = 0; l <= kHidden; ++l) {
    const bool last = l == kHidden;
    const int out_dim = last ? 16 : kMlpH;
    const int kp = tc_k_pad(in_dim), np = tc_n_pad(out_dim);
    const float* bias = reinterpret_cast<const float*>(w + off + kp * np * 2);
    // A complete in every lane -> one thread issues this layer's MMAs
    tc::fence_before_sync();
    tc::tile_sync(T.tile);
    if (issuer) {
      tc::fence_after_sync();
      const uint32_t idesc = tc::idesc_bf16(128, np);
      for (int s = 0; s < kp / 16; ++s) {
        const uint64_t bd = tc::smem_desc(w_saddr + off + s * (np / 8) * 256, kTcLbo, kTcSbo);
        tc::mma_ts(T.tmem_d, T.tmem_a + 8 * s, bd, idesc, s > 0 ? 1u : 0u);
      }
      tc::commit(T.mbar);
    }
    const bool done = tc::tile_all(T.tile, tc::mbar_wait(T.mbar, T.phase, wait_tries));
    T.phase ^= 1u;
    if (!done) return false;  // tile-uniform: stop issuing, leave tensor memory alone
    tc::fence_after_sync();
    if (!last) {
      // SiLU epilogue: D (64 FP32 columns) -> A (32 columns of BF16 pairs)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float v[16];
        tc::ld16(T.tmem_d + lane_off + 16 * c, v);
        uint32_t p[8];
#pragma unroll
        for (int i = 0; i < 8; ++i)
          p[i] = pack_bf16(silu_half(v[2 * i] + bias[16 * c + 2 * i]),
                           silu_half(v[2 * i + 1] + bias[16 * c + 2 * i + 1]));
        tc::st8(T.tmem_a + lane_off + 8 * c, p);
      }
      tc::wait_st();
    } else {
      float v[16];
      tc::ld16(T.tmem_d + lane_off, v);
#pragma unroll
      for (int i = 0; i < 8; ++i) y[i] = v[i] + bias[i];
    }
    off += tc_layer_bytes(in_dim, out_dim);
    in_dim = kMlpH;
  }
  // every lane has read D before the next tile's MMAs overwrite it
  tc::fence_before_sync();
  tc::tile_sync(T.tile);
  return true;
}

}  // namespace atm
