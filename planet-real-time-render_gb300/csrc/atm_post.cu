// atm_post.cu - the display post-process after the atmosphere stage
// (PostProcessor, src/planet_renderer/postprocess.py:75-207) on sm_103a:
// half-resolution bloom extraction with the soft threshold and bright-pass
// cap, separable 5-tap blur passes, and the resolve (exposure, bilinear
// bloom, ACES fit, sRGB).
//
// Memory-bound work: HDR is read twice (extract, resolve) and the display
// written once; the half-resolution bloom planes (float4, W/2 x H/2) stay in
// L2 between the kernels.  A bloom plane is stored with the image's
// contiguous axis fastest, so the extract's HDR reads and writes and the
// resolve's bloom taps are coalesced in either image layout.  Each blur pass
// is one kernel (the reference's two kernels per pass): a 32 x 8 tile of
// output texels loads its 36 x 12 neighbourhood once into shared memory and
// runs the x taps and then the y taps from there, along whichever storage
// axis each lies.  Edge rules are the reference's clamped indices; the clamp
// is applied where the tile is loaded, which gives every tap the texel the
// reference reads.
//
// Arithmetic is IEEE float32 in the reference's operation order with no
// contraction (__fmul_rn / __fadd_rn): every result is the reference's
// float32 result, up to powf's last bit in the sRGB segment.
#include <cuda_runtime.h>

#include <cstdint>

#include "atm_kernels.h"

namespace atm {

namespace {

__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmaxf_(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fminf_(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float clampf_(float x, float lo, float hi) { return fminf_(fmaxf_(x, lo), hi); }

__device__ __forceinline__ float4 scale4(float4 v, float s) {
  return make_float4(mul(v.x, s), mul(v.y, s), mul(v.z, s), 0.0f);
}
__device__ __forceinline__ float4 add4(float4 a, float4 b) {
  return make_float4(add(a.x, b.x), add(a.y, b.y), add(a.z, b.z), 0.0f);
}

// Blur weights, postprocess.py:126-129.
constexpr float kW0 = 0.38774f, kW1 = 0.24477f, kW2 = 0.06136f;

// centre, -1, +1, -2, +2 in the reference's order of summation
__device__ __forceinline__ float4 taps5(float4 c, float4 m1, float4 p1, float4 m2, float4 p2) {
  float4 r = scale4(c, kW0);
  r = add4(r, scale4(m1, kW1));
  r = add4(r, scale4(p1, kW1));
  r = add4(r, scale4(m2, kW2));
  return add4(r, scale4(p2, kW2));
}

__device__ __forceinline__ float4 load_rgb(const float* __restrict__ img, const ImageLayout& L, int x, int y) {
  const float* p = img + (int64_t(x) * L.sx + int64_t(y) * L.sy) * L.channels;
  return make_float4(p[0], p[1], p[2], 0.0f);
}

// _soft_threshold, postprocess.py:88-107.
__device__ __forceinline__ float4 soft_threshold(float4 v, const PostParams& Q) {
  const float brightness = fmaxf_(v.x, fmaxf_(v.y, v.z));
  float soft = clampf_(add(sub(brightness, Q.threshold), Q.knee), 0.0f, Q.two_knee);
  soft = __fdiv_rn(mul(soft, soft), Q.knee_div);
  float contribution = fmaxf_(sub(brightness, Q.threshold), soft);
  contribution = __fdiv_rn(contribution, fmaxf_(brightness, 1.0e-6f));
  float4 r = scale4(v, contribution);
  const float peak = fmaxf_(r.x, fmaxf_(r.y, r.z));
  return scale4(r, fminf_(1.0f, __fdiv_rn(Q.clamp, fmaxf_(peak, 1.0e-6f))));
}

// Storage index of bloom texel (x, y): [y][x] when x is the fast axis, else [x][y].
__device__ __forceinline__ size_t bloom_index(const PostParams& Q, int x, int y) {
  return Q.x_fast ? size_t(y) * Q.hw + x : size_t(x) * Q.hh + y;
}

// _extract, postprocess.py:110-119: one thread per half-resolution texel, in
// storage order.
__global__ void __launch_bounds__(256) k_post_extract(PostParams Q, ImageLayout L, const float* __restrict__ hdr,
                                                      float scale, float4* __restrict__ bloom) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Q.hw * Q.hh) return;
  const int x = Q.x_fast ? i % Q.hw : i / Q.hh;
  const int y = Q.x_fast ? i / Q.hw : i % Q.hh;
  float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int ox = 0; ox < 2; ++ox)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
      v = add4(v, load_rgb(hdr, L, min(2 * x + ox, L.width - 1), min(2 * y + oy, L.height - 1)));
  bloom[i] = soft_threshold(scale4(v, scale), Q);
}

// One blur pass (_blur_horizontal then _blur_vertical, :121-139) fused.  The
// tile is kTileS rows of the slow storage axis by kTileF texels of the fast
// one; kXFast: x (the first pass) runs along the fast axis.
constexpr int kTileF = 32, kTileS = 8, kHalo = 2;
constexpr int kInF = kTileF + 2 * kHalo, kInS = kTileS + 2 * kHalo;

template <bool kXFast>
__global__ void __launch_bounds__(kTileF * kTileS) k_post_blur(PostParams Q, const float4* __restrict__ src,
                                                               float4* __restrict__ dst) {
  __shared__ float4 s_in[kInS][kInF];
  __shared__ float4 s_mid[kInS][kInF];  // after the x taps
  const int t = threadIdx.x;
  const int nf = kXFast ? Q.hw : Q.hh, ns = kXFast ? Q.hh : Q.hw;  // fast / slow extents
  const int f0 = blockIdx.x * kTileF, s0 = blockIdx.y * kTileS;
  for (int k = t; k < kInS * kInF; k += kTileF * kTileS) {
    const int r = k / kInF, c = k % kInF;
    const int gf = min(max(f0 - kHalo + c, 0), nf - 1);
    const int gs = min(max(s0 - kHalo + r, 0), ns - 1);
    s_in[r][c] = src[size_t(gs) * nf + gf];
  }
  __syncthreads();
  if (kXFast) {
    // x taps along the fast axis on every (clamped) slow row, then y taps along the slow axis
    for (int k = t; k < kInS * kTileF; k += kTileF * kTileS) {
      const int r = k / kTileF, c = k % kTileF + kHalo;
      s_mid[r][c] = taps5(s_in[r][c], s_in[r][c - 1], s_in[r][c + 1], s_in[r][c - 2], s_in[r][c + 2]);
    }
  } else {
    // x taps along the slow axis on every (clamped) fast column, then y taps along the fast axis
    for (int k = t; k < kTileS * kInF; k += kTileF * kTileS) {
      const int r = k / kInF + kHalo, c = k % kInF;
      s_mid[r][c] = taps5(s_in[r][c], s_in[r - 1][c], s_in[r + 1][c], s_in[r - 2][c], s_in[r + 2][c]);
    }
  }
  __syncthreads();
  const int c = t % kTileF + kHalo, r = t / kTileF + kHalo;
  const int f = f0 + c - kHalo, sl = s0 + r - kHalo;
  if (f < nf && sl < ns) {
    const float4 out = kXFast ? taps5(s_mid[r][c], s_mid[r - 1][c], s_mid[r + 1][c], s_mid[r - 2][c], s_mid[r + 2][c])
                              : taps5(s_mid[r][c], s_mid[r][c - 1], s_mid[r][c + 1], s_mid[r][c - 2], s_mid[r][c + 2]);
    dst[size_t(sl) * nf + f] = out;
  }
}

// Storage [x][y] -> [y][x] (the bloom plane's read-back).
__global__ void __launch_bounds__(256) k_post_transpose(const float4* __restrict__ src, float4* __restrict__ dst,
                                                        int hw, int hh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hw * hh) return;
  const int x = i % hw, y = i / hw;
  dst[i] = src[size_t(x) * hh + y];
}

// _sample_bloom, postprocess.py:141-153.
__device__ __forceinline__ float4 sample_bloom(const float4* __restrict__ bloom, const PostParams& Q, float u,
                                               float v) {
  const float px = sub(mul(u, float(Q.hw)), 0.5f);
  const float py = sub(mul(v, float(Q.hh)), 0.5f);
  const float fpx = floorf(px), fpy = floorf(py);
  const int x0 = min(max(int(fpx), 0), Q.hw - 1), y0 = min(max(int(fpy), 0), Q.hh - 1);
  const int x1 = min(x0 + 1, Q.hw - 1), y1 = min(y0 + 1, Q.hh - 1);
  const float fx = clampf_(sub(px, fpx), 0.0f, 1.0f), fy = clampf_(sub(py, fpy), 0.0f, 1.0f);
  const float gx = sub(1.0f, fx), gy = sub(1.0f, fy);
  const float4 low = add4(scale4(bloom[bloom_index(Q, x0, y0)], gx), scale4(bloom[bloom_index(Q, x1, y0)], fx));
  const float4 high = add4(scale4(bloom[bloom_index(Q, x0, y1)], gx), scale4(bloom[bloom_index(Q, x1, y1)], fx));
  return add4(scale4(low, gy), scale4(high, fy));
}

// _display_from_exposed, postprocess.py:56-73: ACES fit, sRGB encoding.
__device__ __forceinline__ float display_channel(float v) {
  v = fmaxf_(v, 0.0f);
  const float num = mul(v, add(mul(2.51f, v), 0.03f));
  const float den = add(mul(v, add(mul(2.43f, v), 0.59f)), 0.14f);
  const float mapped = clampf_(__fdiv_rn(num, den), 0.0f, 1.0f);
  if (mapped <= 0.0031308f) return mul(mapped, 12.92f);
  return sub(mul(1.055f, powf(mapped, 0.41666666666666667f)), 0.055f);
}

// _resolve, postprocess.py:155-174: one thread per pixel, threads along the
// image's contiguous axis (Q.x_fast).
__global__ void __launch_bounds__(256) k_post_resolve(PostParams Q, ImageLayout L, const float* __restrict__ hdr,
                                                      float* __restrict__ display, const float4* __restrict__ bloom,
                                                      float exposure, float strength, int use_bloom, int tone_map) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= int64_t(L.width) * L.height) return;
  const int x = Q.x_fast ? int(i % L.width) : int(i / L.height);
  const int y = Q.x_fast ? int(i / L.width) : int(i % L.height);
  float4 v = scale4(load_rgb(hdr, L, x, y), exposure);
  if (use_bloom) {
    const float u = __fdiv_rn(add(float(x), 0.5f), float(L.width));
    const float w = __fdiv_rn(add(float(y), 0.5f), float(L.height));
    v = add4(v, scale4(sample_bloom(bloom, Q, u, w), strength));
  }
  float* out = display + (int64_t(x) * L.sx + int64_t(y) * L.sy) * L.channels;
  if (tone_map) {
    out[0] = display_channel(v.x);
    out[1] = display_channel(v.y);
    out[2] = display_channel(v.z);
  } else {
    out[0] = clampf_(v.x, 0.0f, 1.0f);
    out[1] = clampf_(v.y, 0.0f, 1.0f);
    out[2] = clampf_(v.z, 0.0f, 1.0f);
  }
}

}  // namespace

bool image_x_fast(const ImageLayout& L) {
  const int64_t ax = L.sx < 0 ? -L.sx : L.sx, ay = L.sy < 0 ? -L.sy : L.sy;
  return ax < ay;
}

cudaError_t launch_post(const PostParams& Q, const ImageLayout& L, const float* hdr, float* display, float4* bloom_a,
                        float4* bloom_b, float exposure, float strength, int passes, bool use_bloom, bool tone_map,
                        const float4** bloom_out, cudaStream_t s) {
  const float4* bloom = bloom_a;
  if (use_bloom) {
    const int n = Q.hw * Q.hh;
    k_post_extract<<<(n + 255) / 256, 256, 0, s>>>(Q, L, hdr, 0.25f * exposure, bloom_a);  // exact: a power of two
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int nf = Q.x_fast ? Q.hw : Q.hh, ns = Q.x_fast ? Q.hh : Q.hw;
    const dim3 grid((nf + kTileF - 1) / kTileF, (ns + kTileS - 1) / kTileS);
    float4* src = bloom_a;
    float4* dst = bloom_b;
    for (int p = 0; p < passes; ++p) {
      if (Q.x_fast)
        k_post_blur<true><<<grid, kTileF * kTileS, 0, s>>>(Q, src, dst);
      else
        k_post_blur<false><<<grid, kTileF * kTileS, 0, s>>>(Q, src, dst);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      float4* tmp = src;
      src = dst;
      dst = tmp;
    }
    bloom = src;
  }
  if (bloom_out != nullptr) *bloom_out = bloom;
  const int64_t pixels = int64_t(L.width) * L.height;
  k_post_resolve<<<unsigned((pixels + 255) / 256), 256, 0, s>>>(Q, L, hdr, display, bloom, exposure, strength,
                                                                 use_bloom ? 1 : 0, tone_map ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_post_read_bloom(const PostParams& Q, const float4* bloom, float4* dst, cudaStream_t s) {
  const size_t n = size_t(Q.hw) * Q.hh;
  if (Q.x_fast) return cudaMemcpyAsync(dst, bloom, n * sizeof(float4), cudaMemcpyDeviceToDevice, s);
  k_post_transpose<<<unsigned((n + 255) / 256), 256, 0, s>>>(bloom, dst, Q.hw, Q.hh);
  return cudaGetLastError();
}

}  // namespace atm
