// atm_mlp.cu - small MLP surrogates: fused FP32 training (forward + backward)
// on CUDA cores, Adam, an FP32 reference forward and a BF16 tensor-core
// forward (mma.sync m16n8k16, FP32 accumulate).
//
// Network: n_in -> [64 SiLU] x n_hidden -> n_out (n_in <= 16, n_out <= 8,
// n_hidden 1..4).  Parameters are one float array: for each layer l, W_l
// (out x in, row-major) then b_l.  The training objective is the mean
// squared error over all outputs of the batch.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "atm_kernels.h"
#include "atm_mlp_tc.cuh"
#include "atm_mlp_tile.cuh"

namespace atm {

namespace {

constexpr int kH = 64;          // hidden width
constexpr int kS = 64;          // samples per training CTA
constexpr int kThreads = 256;
constexpr int kStride = kH + 1; // padded smem row of a 64-wide activation

__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }
// The training kernel's sigmoid: the hardware exponential and reciprocal
// (a few ulp; the gradients are checked against the FP64 oracle at 1e-4).
__device__ __forceinline__ float sigmoid_fast(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }

// Shared-memory layout of the training kernel (float offsets).
struct TrainSmem {
  int w[kMaxMlpLayers], b[kMaxMlpLayers];  // weights [out][in+1], biases
  int x;                                   // inputs [kS][n_in+1]
  int z[kMaxMlpLayers], a[kMaxMlpLayers];  // hidden pre-/post-activations [kS][65]
  int y;                                   // outputs / output gradients [kS][n_out+1]
  int total;
};

__host__ __device__ inline TrainSmem train_smem(const MlpShape& m) {
  TrainSmem t{};
  int o = 0;
  for (int l = 0; l < m.n_layers; ++l) {
    t.w[l] = o;
    o += m.out_dim[l] * (m.in_dim[l] + 1);
    t.b[l] = o;
    o += m.out_dim[l];
  }
  t.x = o;
  o += kS * (m.n_in + 1);
  for (int l = 0; l + 1 < m.n_layers; ++l) {
    t.z[l] = o;
    o += kS * kStride;
    t.a[l] = o;
    o += kS * kStride;
  }
  t.y = o;
  o += kS * (m.n_out + 1);
  t.total = o;
  return t;
}

// out[s][j] = b[j] + sum_k in[s][k] W[j][k] for s < kS, j < out_dim.
// 64-wide outputs: a thread holds 4 samples x 4 columns j0 + 16c (columns
// interleaved so that a warp's weight reads hit distinct banks).
__device__ void dense_forward(const float* __restrict__ in, int in_stride, int in_dim, const float* __restrict__ W,
                              const float* __restrict__ b, int out_dim, float* __restrict__ out, int out_stride) {
  const int t = threadIdx.x;
  if (out_dim == kH) {
    const int s0 = (t >> 4) * 4, j0 = t & 15;
    float acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c] = b[j0 + 16 * c];
    for (int k = 0; k < in_dim; ++k) {
      float av[4], wv[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) av[r] = in[(s0 + r) * in_stride + k];
#pragma unroll
      for (int c = 0; c < 4; ++c) wv[c] = W[(j0 + 16 * c) * (in_dim + 1) + k];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(av[r], wv[c], acc[r][c]);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) out[(s0 + r) * out_stride + j0 + 16 * c] = acc[r][c];
  } else {
    for (int idx = t; idx < kS * out_dim; idx += kThreads) {
      const int s = idx / out_dim, j = idx % out_dim;
      float acc = b[j];
      for (int k = 0; k < in_dim; ++k) acc = fmaf(in[s * in_stride + k], W[j * (in_dim + 1) + k], acc);
      out[s * out_stride + j] = acc;
    }
  }
}

// Fused forward + backward over one tile of kS samples; writes this CTA's
// gradient of the batch loss (every parameter) and its squared-error sum.
__global__ void __launch_bounds__(kThreads) k_mlp_grad(MlpShape m, const float* __restrict__ params,
                                                       const float* __restrict__ inputs,
                                                       const float* __restrict__ targets,
                                                       const float* __restrict__ weights, long long n,
                                                       float inv_count, float* __restrict__ grad_partial,
                                                       float* __restrict__ loss_partial) {
  extern __shared__ float sm[];
  const TrainSmem L = train_smem(m);
  const int t = threadIdx.x;
  const long long base = static_cast<long long>(blockIdx.x) * kS;
  const int L_out = m.n_layers - 1;
  // weights and biases -> smem (padded rows)
  for (int l = 0; l < m.n_layers; ++l) {
    const int in = m.in_dim[l], out = m.out_dim[l];
    for (int i = t; i < out * in; i += kThreads) sm[L.w[l] + (i / in) * (in + 1) + i % in] = params[m.off_w[l] + i];
    for (int i = t; i < out; i += kThreads) sm[L.b[l] + i] = params[m.off_b[l] + i];
  }
  for (int i = t; i < kS * m.n_in; i += kThreads) {
    const int s = i / m.n_in, k = i % m.n_in;
    sm[L.x + s * (m.n_in + 1) + k] = base + s < n ? inputs[(base + s) * m.n_in + k] : 0.0f;
  }
  __syncthreads();
  // forward
  for (int l = 0; l < m.n_layers; ++l) {
    const float* in = l == 0 ? sm + L.x : sm + L.a[l - 1];
    const int in_stride = l == 0 ? m.n_in + 1 : kStride;
    float* out = l == L_out ? sm + L.y : sm + L.z[l];
    const int out_stride = l == L_out ? m.n_out + 1 : kStride;
    dense_forward(in, in_stride, m.in_dim[l], sm + L.w[l], sm + L.b[l], m.out_dim[l], out, out_stride);
    __syncthreads();
    if (l != L_out) {
      for (int i = t; i < kS * kH; i += kThreads) {
        const int s = i / kH, j = i % kH;
        const float z = sm[L.z[l] + s * kStride + j];
        sm[L.a[l] + s * kStride + j] = z * sigmoid_fast(z);
      }
      __syncthreads();
    }
  }
  // loss and output gradient (mean over batch x outputs)
  float sq = 0.0f;
  for (int i = t; i < kS * m.n_out; i += kThreads) {
    const int s = i / m.n_out, o = i % m.n_out;
    float g = 0.0f;
    if (base + s < n) {
      const float d = sm[L.y + s * (m.n_out + 1) + o] - targets[(base + s) * m.n_out + o];
      const float w = weights != nullptr ? weights[(base + s) * m.n_out + o] : 1.0f;
      sq += w * d * d;
      g = 2.0f * w * d * inv_count;
    }
    sm[L.y + s * (m.n_out + 1) + o] = g;
  }
  __syncthreads();
  // backward: dZ_l lives in place of Z_l (or Y for the output layer)
  float* gp = grad_partial + static_cast<long long>(blockIdx.x) * m.n_params;
  for (int l = L_out; l >= 0; --l) {
    const int in = m.in_dim[l], out = m.out_dim[l];
    const float* dz = l == L_out ? sm + L.y : sm + L.z[l];
    const int dz_stride = l == L_out ? m.n_out + 1 : kStride;
    const float* a_prev = l == 0 ? sm + L.x : sm + L.a[l - 1];
    const int a_stride = l == 0 ? m.n_in + 1 : kStride;
    // dW[j][k] = sum_s dz[s][j] a_prev[s][k];  db[j] = sum_s dz[s][j]
    if (out == kH) {
      // register tiles: 4 neurons j = 4 (t >> 4) + r by in/16 inputs
      // k = (t & 15) + 16 c; per sample 8 shared loads feed 16 FMAs
      const int j0 = (t >> 4) * 4, kk = t & 15;
      float acc[4][4] = {};
      float bacc = 0.0f;
      for (int s = 0; s < kS; ++s) {
        float dv[4], av[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) dv[r] = dz[s * dz_stride + j0 + r];
#pragma unroll
        for (int c = 0; c < 4; ++c) av[c] = kk + 16 * c < in ? a_prev[s * a_stride + kk + 16 * c] : 0.0f;
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(dv[r], av[c], acc[r][c]);
        bacc += kk == 0 ? dv[0] : kk == 1 ? dv[1] : kk == 2 ? dv[2] : dv[3];  // used by kk < 4
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (kk + 16 * c < in) gp[m.off_w[l] + (j0 + r) * in + kk + 16 * c] = acc[r][c];
      if (kk < 4) gp[m.off_b[l] + j0 + kk] = bacc;
    } else {
      for (int idx = t; idx < out * in; idx += kThreads) {
        const int j = idx / in, k = idx % in;
        float acc = 0.0f;
        for (int s = 0; s < kS; ++s) acc = fmaf(dz[s * dz_stride + j], a_prev[s * a_stride + k], acc);
        gp[m.off_w[l] + idx] = acc;
      }
      for (int j = t; j < out; j += kThreads) {
        float acc = 0.0f;
        for (int s = 0; s < kS; ++s) acc += dz[s * dz_stride + j];
        gp[m.off_b[l] + j] = acc;
      }
    }
    if (l == 0) break;
    // dZ_{l-1}[s][k] = (sum_j dz[s][j] W[j][k]) * silu'(Z_{l-1}[s][k]), in
    // place of Z_{l-1} (in == 64 here): register tiles of 4 samples
    // s = 4 (t >> 4) + r by 4 inputs k = (t & 15) + 16 c
    const float* W = sm + L.w[l];
    float* zp = sm + L.z[l - 1];
    const int s0 = (t >> 4) * 4, kk = t & 15;
    float acc[4][4] = {};
    for (int j = 0; j < out; ++j) {
      float dv[4], wv[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) dv[r] = dz[(s0 + r) * dz_stride + j];
#pragma unroll
      for (int c = 0; c < 4; ++c) wv[c] = W[j * (in + 1) + kk + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(dv[r], wv[c], acc[r][c]);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float z = zp[(s0 + r) * kStride + kk + 16 * c];
        const float sg = sigmoid_fast(z);
        acc[r][c] = acc[r][c] * sg * (1.0f + z * (1.0f - sg));
      }
    __syncthreads();  // all reads of Z_{l-1} (and of dZ_l by the dW loop) are done
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) zp[(s0 + r) * kStride + kk + 16 * c] = acc[r][c];
    __syncthreads();
  }
  // squared-error sum of the tile
  __shared__ float s_red[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  if ((t & 31) == 0) s_red[t >> 5] = sq;
  __syncthreads();
  if (t == 0) {
    float total = 0.0f;
    for (int w = 0; w < kThreads / 32; ++w) total += s_red[w];
    loss_partial[blockIdx.x] = total;
  }
}

// grad[p] = sum over CTAs of grad_partial[cta][p], in CTA order.
__global__ void k_reduce_partials(const float* __restrict__ partial, int n_ctas, int n_params,
                                  float* __restrict__ out) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_params; p += gridDim.x * blockDim.x) {
    float acc = 0.0f;
    for (int c = 0; c < n_ctas; ++c) acc += partial[static_cast<long long>(c) * n_params + p];
    out[p] = acc;
  }
}

__global__ void k_adam(float* __restrict__ params, const float* __restrict__ grad, float* __restrict__ m1,
                       float* __restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const float g = grad[p];
    const float a = b1 * m1[p] + (1.0f - b1) * g;
    const float v = b2 * m2[p] + (1.0f - b2) * g * g;
    m1[p] = a;
    m2[p] = v;
    params[p] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
  }
}

// FP32 forward, one thread per sample (reference path of the BF16 kernel).
__global__ void __launch_bounds__(128) k_mlp_forward_f32(MlpShape m, const float* __restrict__ params,
                                                        const float* __restrict__ inputs, float* __restrict__ outputs,
                                                        long long n) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  float a[kH], z[kH];
  for (int k = 0; k < m.n_in; ++k) a[k] = inputs[i * m.n_in + k];
  for (int l = 0; l < m.n_layers; ++l) {
    const float* W = params + m.off_w[l];
    const float* b = params + m.off_b[l];
    const int in = m.in_dim[l], out = m.out_dim[l];
    for (int j = 0; j < out; ++j) {
      float acc = b[j];
      for (int k = 0; k < in; ++k) acc = fmaf(a[k], __ldg(W + j * in + k), acc);
      z[j] = acc;
    }
    if (l + 1 == m.n_layers) {
      for (int j = 0; j < out; ++j) outputs[i * m.n_out + j] = z[j];
    } else {
      for (int j = 0; j < out; ++j) a[j] = z[j] * sigmoid(z[j]);
    }
  }
}

}  // namespace

// Byte size of the packed BF16 network.
size_t mlp_bf16_bytes(const MlpShape& m) {
  size_t bytes = 0;
  for (int l = 0; l < m.n_layers; ++l) {
    const int op = mlp_bf16_out_pad(m.out_dim[l]);
    bytes += size_t(op) * mlp_bf16_layer_row(m.in_dim[l]) * 2;
    bytes += size_t(op) * 4;
  }
  return bytes;
}

namespace {

// Hidden layers are stored with W and b halved (exact in BF16), so their
// accumulators hold z / 2 for the packed SiLU of mlp_tile_bf16.
__global__ void k_pack_bf16(MlpShape m, const float* __restrict__ params, unsigned char* __restrict__ packed) {
  size_t off = 0;
  for (int l = 0; l < m.n_layers; ++l) {
    const int in = m.in_dim[l], out = m.out_dim[l];
    const int row = mlp_bf16_layer_row(in), op = mlp_bf16_out_pad(out);
    const float scale = l + 1 < m.n_layers ? 0.5f : 1.0f;
    __nv_bfloat16* W = reinterpret_cast<__nv_bfloat16*>(packed + off);
    for (int i = threadIdx.x; i < op * row; i += blockDim.x) {
      const int j = i / row, k = i % row;
      const float v = (j < out && k < in) ? params[m.off_w[l] + j * in + k] : 0.0f;
      W[i] = __float2bfloat16_rn(v * scale);
    }
    off += size_t(op) * row * 2;
    float* b = reinterpret_cast<float*>(packed + off);
    for (int j = threadIdx.x; j < op; j += blockDim.x) b[j] = j < out ? params[m.off_b[l] + j] * scale : 0.0f;
    off += size_t(op) * 4;
  }
}

// tcgen05 layout of a network (atm_mlp_tc.cuh): weights as K-major core
// matrices, hidden layers halved.
__global__ void k_pack_tc(MlpShape m, const float* __restrict__ params, unsigned char* __restrict__ packed) {
  int off = 0;
  for (int l = 0; l < m.n_layers; ++l) {
    const int in = m.in_dim[l], out = m.out_dim[l];
    const int kp = tc_k_pad(in), np = tc_n_pad(out);
    const float scale = l + 1 < m.n_layers ? 0.5f : 1.0f;
    for (int i = threadIdx.x; i < kp * np; i += blockDim.x) {
      const int n = i / kp, k = i % kp;
      const float v = (n < out && k < in) ? params[m.off_w[l] + n * in + k] * scale : 0.0f;
      *reinterpret_cast<__nv_bfloat16*>(packed + off + tc_w_offset(n, k, np)) = __float2bfloat16_rn(v);
    }
    float* b = reinterpret_cast<float*>(packed + off + kp * np * 2);
    for (int j = threadIdx.x; j < np; j += blockDim.x) b[j] = j < out ? params[m.off_b[l] + j] * scale : 0.0f;
    off += tc_layer_bytes(in, out);
  }
}

// Forward of n samples on the tcgen05 path: one tile of 128 samples per
// block at a time (grid-stride); TMEM: accumulators at column 0, activations
// at column 128 of a 256-column allocation.  *error is set when an MMA did
// not complete in time.
template <int kHidden>
__global__ void __launch_bounds__(128) k_mlp_forward_tc(MlpShape m, const unsigned char* __restrict__ packed,
                                                        int packed_bytes, const float* __restrict__ inputs,
                                                        float* __restrict__ outputs, long long n,
                                                        int* __restrict__ error) {
  extern __shared__ __align__(128) unsigned char smw[];
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ uint32_t s_tmem;
  for (int i = threadIdx.x * 16; i < packed_bytes; i += blockDim.x * 16)
    *reinterpret_cast<uint4*>(smw + i) = *reinterpret_cast<const uint4*>(packed + i);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> tensor-core reads
  if (threadIdx.x < 32) tc::alloc(&s_tmem, 256);
  if (threadIdx.x == 0) {
    tc::mbar_init(&s_mbar, 1);
    tc::mbar_init_fence();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  TcTile T{s_tmem, s_tmem + 128, &s_mbar, 0u, 0, int(threadIdx.x)};
  bool ok = true;
  for (long long base = blockIdx.x * 128LL; base < n; base += gridDim.x * 128LL) {
    const long long r = base + threadIdx.x;
    float x[16] = {}, y[8];
    if (r < n)
      for (int k = 0; k < m.n_in; ++k) x[k] = inputs[r * m.n_in + k];
    ok = mlp_tile_tc<kHidden>(smw, m.n_in, T, x, y);
    if (!ok) break;  // block-uniform (one tile per block); no MMA is issued after it
    if (r < n)
      for (int k = 0; k < m.n_out; ++k) outputs[r * m.n_out + k] = y[k];
  }
  if (!ok && threadIdx.x == 0) atomicExch(error, 1);
  // before the tensor memory is freed, no MMA of this CTA may be in flight:
  // after a timed-out wait, wait once more (bounded) for its one commit
  tc::fence_before_sync();
  if (__syncthreads_or(!ok)) tc::mbar_wait(&s_mbar, T.phase ^ 1u, kTcWaitTries);
  __syncthreads();
  tc::fence_after_sync();
  if (threadIdx.x < 32) tc::dealloc(s_tmem, 256);
}

template <int kHidden>
__global__ void __launch_bounds__(128) k_mlp_forward_bf16(MlpShape m, const unsigned char* __restrict__ packed,
                                                          int packed_bytes, const float* __restrict__ inputs,
                                                          float* __restrict__ outputs, long long n) {
  extern __shared__ __align__(16) unsigned char smw[];
  for (int i = threadIdx.x * 4; i < packed_bytes; i += blockDim.x * 4)
    *reinterpret_cast<uint32_t*>(smw + i) = *reinterpret_cast<const uint32_t*>(packed + i);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, q = lane & 3;
  const int in0_row = mlp_bf16_layer_row(m.n_in);
  const long long warps = static_cast<long long>(gridDim.x) * (blockDim.x >> 5);
  for (long long tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n; tile += warps) {
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
    auto in = [&](long long r, int k) { return (r < n && k < m.n_in) ? inputs[r * m.n_in + k] : 0.0f; };
    uint32_t x[4];
    x[0] = pack_bf16(in(r0, 2 * q), in(r0, 2 * q + 1));
    x[1] = pack_bf16(in(r1, 2 * q), in(r1, 2 * q + 1));
    x[2] = pack_bf16(in(r0, 8 + 2 * q), in(r0, 8 + 2 * q + 1));
    x[3] = pack_bf16(in(r1, 8 + 2 * q), in(r1, 8 + 2 * q + 1));
    float y[4];
    mlp_tile_bf16<kHidden>(smw, x, in0_row, y);
    for (int i = 0; i < 2; ++i) {
      const int o = 2 * q + i;
      if (o < m.n_out) {
        if (r0 < n) outputs[r0 * m.n_out + o] = y[i];
        if (r1 < n) outputs[r1 * m.n_out + o] = y[2 + i];
      }
    }
  }
}

}  // namespace

MlpShape make_mlp_shape(int n_in, int n_hidden, int n_out) {
  MlpShape m{};
  m.n_in = n_in;
  m.n_out = n_out;
  m.n_layers = n_hidden + 1;
  int off = 0;
  for (int l = 0; l < m.n_layers; ++l) {
    m.in_dim[l] = l == 0 ? n_in : kH;
    m.out_dim[l] = l == n_hidden ? n_out : kH;
    m.off_w[l] = off;
    off += m.in_dim[l] * m.out_dim[l];
    m.off_b[l] = off;
    off += m.out_dim[l];
  }
  m.n_params = off;
  return m;
}

int mlp_train_ctas(long long n) { return int((n + kS - 1) / kS); }

size_t mlp_train_smem_bytes(const MlpShape& m) { return size_t(train_smem(m).total) * sizeof(float); }

cudaError_t launch_mlp_grad(const MlpShape& m, const float* params, const float* inputs, const float* targets,
                            const float* weights, long long n, float* grad_partial, float* loss_partial, float* grad,
                            cudaStream_t s) {
  const size_t smem = mlp_train_smem_bytes(m);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return e;
  const int ctas = mlp_train_ctas(n);
  const float inv = 1.0f / float(double(n) * m.n_out);
  k_mlp_grad<<<ctas, kThreads, smem, s>>>(m, params, inputs, targets, weights, n, inv, grad_partial, loss_partial);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_reduce_partials<<<(m.n_params + 255) / 256, 256, 0, s>>>(grad_partial, ctas, m.n_params, grad);
  return cudaGetLastError();
}

cudaError_t launch_reduce_partials(const float* partial, int rows, int cols, float* out, cudaStream_t s) {
  k_reduce_partials<<<(cols + 255) / 256, 256, 0, s>>>(partial, rows, cols, out);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* params, const float* grad, float* m1, float* m2, int n, float lr, float b1, float b2,
                        float eps, long long step, cudaStream_t s) {
  const float c1 = 1.0f - float(pow(double(b1), double(step)));
  const float c2 = 1.0f - float(pow(double(b2), double(step)));
  k_adam<<<(n + 255) / 256, 256, 0, s>>>(params, grad, m1, m2, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t launch_mlp_forward_f32(const MlpShape& m, const float* params, const float* inputs, float* outputs,
                                   long long n, cudaStream_t s) {
  k_mlp_forward_f32<<<unsigned((n + 127) / 128), 128, 0, s>>>(m, params, inputs, outputs, n);
  return cudaGetLastError();
}

size_t mlp_tc_bytes(const MlpShape& m) {
  size_t b = 0;
  for (int l = 0; l < m.n_layers; ++l) b += size_t(tc_layer_bytes(m.in_dim[l], m.out_dim[l]));
  return b;
}

cudaError_t launch_mlp_pack_tc(const MlpShape& m, const float* params, void* packed, cudaStream_t s) {
  k_pack_tc<<<1, 256, 0, s>>>(m, params, static_cast<unsigned char*>(packed));
  return cudaGetLastError();
}

cudaError_t launch_mlp_forward_tc(const MlpShape& m, const void* packed, const float* inputs, float* outputs,
                                  long long n, int* error, int sm_count, cudaStream_t s) {
  const int bytes = int(mlp_tc_bytes(m));
  const unsigned blocks = unsigned(std::min<long long>((n + 127) / 128, 2LL * sm_count));
  const auto* p = static_cast<const unsigned char*>(packed);
  cudaError_t e = cudaSuccess;
  switch (m.n_layers - 1) {
    case 1: e = cudaFuncSetAttribute(k_mlp_forward_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
      if (e == cudaSuccess) k_mlp_forward_tc<1><<<blocks, 128, bytes, s>>>(m, p, bytes, inputs, outputs, n, error);
      break;
    case 2: e = cudaFuncSetAttribute(k_mlp_forward_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
      if (e == cudaSuccess) k_mlp_forward_tc<2><<<blocks, 128, bytes, s>>>(m, p, bytes, inputs, outputs, n, error);
      break;
    case 3: e = cudaFuncSetAttribute(k_mlp_forward_tc<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
      if (e == cudaSuccess) k_mlp_forward_tc<3><<<blocks, 128, bytes, s>>>(m, p, bytes, inputs, outputs, n, error);
      break;
    case 4: e = cudaFuncSetAttribute(k_mlp_forward_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
      if (e == cudaSuccess) k_mlp_forward_tc<4><<<blocks, 128, bytes, s>>>(m, p, bytes, inputs, outputs, n, error);
      break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_mlp_pack_bf16(const MlpShape& m, const float* params, void* packed, cudaStream_t s) {
  k_pack_bf16<<<1, 256, 0, s>>>(m, params, static_cast<unsigned char*>(packed));
  return cudaGetLastError();
}

cudaError_t launch_mlp_forward_bf16(const MlpShape& m, const void* packed, const float* inputs, float* outputs,
                                    long long n, int sm_count, cudaStream_t s) {
  const int bytes = int(mlp_bf16_bytes(m));
  const unsigned blocks = unsigned(std::min<long long>((n + 63) / 64, 8LL * sm_count));
  const auto* p = static_cast<const unsigned char*>(packed);
  switch (m.n_layers - 1) {
    case 1: k_mlp_forward_bf16<1><<<blocks, 128, bytes, s>>>(m, p, bytes, inputs, outputs, n); break;
    case 2: k_mlp_forward_bf16<2><<<blocks, 128, bytes, s>>>(m, p, bytes, inputs, outputs, n); break;
    case 3: k_mlp_forward_bf16<3><<<blocks, 128, bytes, s>>>(m, p, bytes, inputs, outputs, n); break;
    case 4: k_mlp_forward_bf16<4><<<blocks, 128, bytes, s>>>(m, p, bytes, inputs, outputs, n); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace atm
