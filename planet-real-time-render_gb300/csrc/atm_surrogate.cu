// atm_surrogate.cu - learned surrogates of the sky radiance and of the
// camera-to-surface in-scattering / transmittance.
//
//  * k_gen_samples: training samples produced by the plain integrator itself
//    (the same device functions as the LUT builds and the composite).
//  * k_composite_surrogate: the COMPOSITE view with the per-pixel limb
//    integrator (renderer.py :1667-1786) replaced by a BF16 tensor-core MLP,
//    and optionally the sky-view lookup by a second MLP; the plain integrator
//    remains the per-pixel fallback where a gate trips (limb, twilight) and
//    re-integrates a random fraction of pixels to measure the MLP's error.
//
// Geometry is reparameterised exactly: the atmosphere is spherically
// symmetric, so a segment is described by the altitude of its first point
// inside the shell, the view and sun cosines there, their relative azimuth
// and its length.  Features use the reference's own horizon-concentrating
// coordinates (sky-view v, multi-scattering u) so that the limb and the
// terminator get the same resolution the LUTs give them.
#include <cuda_runtime.h>

#include <cstdint>

#include "atm_device.cuh"
#include "atm_frame_paths.cuh"
#include "atm_kernels.h"
#include "atm_mlp_tile.cuh"

namespace atm {

namespace {

constexpr unsigned kAll = 0xffffffffu;

__host__ __device__ inline float norm_log(float v, float lo, float hi) {
  return 2.0f * (logf(v) - logf(lo)) / (logf(hi) - logf(lo)) - 1.0f;
}

// x[0..3]: altitude, view, sun, relative azimuth at the segment's first point.
__device__ __forceinline__ void geometry_features(const DevParams& P, float bottom, float h, float mu_v, float mu_s,
                                                  float cos_dphi, float* x) {
  const float hn = clampf(h * P.inv_top, 0.0f, 1.0f);
  x[0] = 2.0f * sqrtf(hn) - 1.0f;
  x[1] = 2.0f * sky_zenith_to_v(acosf(clampf(mu_v, -1.0f, 1.0f)), sky_horizon_zenith(h, bottom)) - 1.0f;
  x[2] = 2.0f * sun_cosine_to_u(clampf(mu_s, -1.0f, 1.0f), horizon_cosine(h, bottom)) - 1.0f;
  x[3] = clampf(cos_dphi, -1.0f, 1.0f);
}

// Counter-based uniform in [0, 1): 64-bit mix of (seed, index, lane).
__device__ __forceinline__ float uniform01(unsigned long long seed, unsigned long long i, unsigned k) {
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (i * 16 + k + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return float(z >> 40) * (1.0f / 16777216.0f);
}

// Sky radiance along `ray` from altitude h (the sky-view march, one thread).
__device__ f3 sky_radiance(const DevParams& P, const Frame& F, float h, f3 ray) {
  float start, end;
  bool valid, ground;
  segment_from_altitude(P, h, ray.y, F.bottom, start, end, valid, ground);
  Seg acc = {splat(0.0f), splat(1.0f)};
  if (valid) {
    const float o_y = F.bottom + h;
    const RaySource rs = make_ray_source(P, F, o_y, h, ray);
    const RayWarp rw = make_warp(-(o_y * ray.y), start, end);
    const int n = P.sv_steps;
    float d0 = warp_at(rw, 0.0f);
    for (int i = 0; i < n; ++i) {
      const float d1 = warp_at(rw, float(i + 1) / float(n));
      float vis;
      acc = seg_then(acc, source_segment<true>(P, F, rs, d0, d1, vis));
      d0 = d1;
    }
  }
  return vmax(acc.L, 0.0f);
}

__global__ void __launch_bounds__(128) k_gen_samples(const SurrogateSetDev* __restrict__ sets, int n_sets, int kind,
                                                     long long n, unsigned long long seed, f3 E, float ar,
                                                     float* __restrict__ features, float* __restrict__ targets,
                                                     unsigned long long* __restrict__ counter) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  uint32_t samples = 0;
  if (i < n) {
    const SurrogateSetDev& S = sets[min(int(uniform01(seed, i, 0) * n_sets), n_sets - 1)];
    const DevParams& P = S.P;
    const float R = S.bottom;
    float x[8];
    for (int k = 0; k < 4; ++k) x[k] = 2.0f * uniform01(seed, i, k + 1) - 1.0f;
    // invert the feature maps
    const float h = P.top * 0.25f * (x[0] + 1.0f) * (x[0] + 1.0f);
    const float zen = sky_v_to_zenith(0.5f * (x[1] + 1.0f), sky_horizon_zenith(h, R));
    float sv, mu_v;
    sincosf(zen, &sv, &mu_v);
    const float mu_s = sun_u_to_cosine(0.5f * (x[2] + 1.0f), h, R);
    const float ss = sqrtf(mx(1.0f - mu_s * mu_s, 0.0f));
    const float cphi = x[3], sphi = sqrtf(mx(1.0f - cphi * cphi, 0.0f));
    const f3 ray = mk(sv, mu_v, 0.0f);
    const f3 sun = mk(ss * cphi, mu_s, ss * sphi);
    geometry_features(P, R, h, mu_v, mu_s, cphi, x);  // rounding-consistent features
    x[4] = S.lhr_n;
    x[5] = S.lhm_n;
    const Frame F = make_frame(P, S.tlut, S.mslut, R, ar, sun, E);
    const f3 inv_e = mk(1.0f / E.x, 1.0f / E.y, 1.0f / E.z);
    if (kind == 0) {  // sky: 6 features -> log(L/E + floor)
      const f3 L = sky_radiance(P, F, h, ray) * inv_e;
      samples = uint32_t(P.sv_steps);
      for (int k = 0; k < 6; ++k) features[i * 6 + k] = x[k];
      targets[i * 3 + 0] = logf(L.x + kSurrogateFloor);
      targets[i * 3 + 1] = logf(L.y + kSurrogateFloor);
      targets[i * 3 + 2] = logf(L.z + kSurrogateFloor);
    } else {  // aerial: + log length -> log(L/E + floor), optical depth
      const float u = uniform01(seed, i, 5);
      const float len = expf(u * logf(kSurrogateMaxLength));
      x[6] = 2.0f * u - 1.0f;
      f3 L = splat(0.0f), T = splat(1.0f);
      float start, end;
      if (surface_interval(P, h, mu_v, R, len, start, end)) {
        L = integrate_surface(P, F, h, ray, start, end, samples) * inv_e;
        T = surface_segment_t(P, F, h, ray, start, end);
      }
      for (int k = 0; k < 7; ++k) features[i * 7 + k] = x[k];
      targets[i * 6 + 0] = logf(L.x + kSurrogateFloor);
      targets[i * 6 + 1] = logf(L.y + kSurrogateFloor);
      targets[i * 6 + 2] = logf(L.z + kSurrogateFloor);
      targets[i * 6 + 3] = mn(-logf(mx(T.x, 1.0e-30f)), kSurrogateMaxDepth);
      targets[i * 6 + 4] = mn(-logf(mx(T.y, 1.0e-30f)), kSurrogateMaxDepth);
      targets[i * 6 + 5] = mn(-logf(mx(T.z, 1.0e-30f)), kSurrogateMaxDepth);
    }
  }
  warp_count(samples, counter);
}

// Lane `src`'s packed feature pair q of this lane's quad position.
__device__ __forceinline__ uint32_t gather_pair(const uint32_t (&xp)[4], int src, int q) {
  uint32_t v0 = __shfl_sync(kAll, xp[0], src), v1 = __shfl_sync(kAll, xp[1], src);
  uint32_t v2 = __shfl_sync(kAll, xp[2], src), v3 = __shfl_sync(kAll, xp[3], src);
  return q == 0 ? v0 : (q == 1 ? v1 : (q == 2 ? v2 : v3));
}

// Evaluates a network on the warp's 32 pixels (two 16-row tiles; every lane
// must call).  x: this lane's 8 features; out: this lane's outputs 0..7.
template <int kHidden>
__device__ __forceinline__ void warp_mlp(const unsigned char* __restrict__ w, int in0_row, const float (&x)[8],
                                         float (&out)[8]) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, q = lane & 3;
  uint32_t xp[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) xp[k] = pack_bf16(x[2 * k], x[2 * k + 1]);
#pragma unroll
  for (int tile = 0; tile < 2; ++tile) {
    const uint32_t frag[4] = {gather_pair(xp, tile * 16 + g, q), gather_pair(xp, tile * 16 + g + 8, q), 0u, 0u};
    float y[4];
    mlp_tile_bf16<kHidden>(w, frag, in0_row, y);
    // row r of this tile lives in lanes (r % 8) * 4 + c/2, registers (r >= 8) * 2 + c % 2
    const int r = lane & 15;
    const bool mine = (lane >> 4) == tile;
#pragma unroll
    for (int cp = 0; cp < 4; ++cp) {
      const int src = (r & 7) * 4 + cp;
      const float lo = __shfl_sync(kAll, y[0], src), hi = __shfl_sync(kAll, y[1], src);
      const float lo8 = __shfl_sync(kAll, y[2], src), hi8 = __shfl_sync(kAll, y[3], src);
      if (mine) {
        out[2 * cp] = r >= 8 ? lo8 : lo;
        out[2 * cp + 1] = r >= 8 ? hi8 : hi;
      }
    }
  }
}

__device__ __forceinline__ bool check_pixel(int x, int y, unsigned seed, float fraction) {
  unsigned h = (unsigned(x) * 0x8DA6B343u) ^ (unsigned(y) * 0xD8163841u) ^ (seed * 0x9E3779B1u);
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  return float(h >> 8) * (1.0f / 16777216.0f) < fraction;
}

__global__ void __launch_bounds__(256, 2) k_composite_surrogate(
    DevParams P, ImageLayout L, CompositeScalars A, const float* __restrict__ scene, const float* __restrict__ space,
    const int32_t* __restrict__ sid, const float* __restrict__ pos, const float4* __restrict__ tlut,
    const float4* __restrict__ mslut, const float4* __restrict__ svlut, SurrogateNets nets, unsigned seed,
    float check_fraction, float* __restrict__ hdr, float* __restrict__ stats, unsigned long long* counter) {
  extern __shared__ __align__(16) unsigned char sw[];
  const int total = nets.ap_bytes + nets.sky_bytes;
  for (int i = threadIdx.x * 4; i < total; i += blockDim.x * 4) {
    const unsigned char* src = i < nets.ap_bytes ? nets.ap + i : nets.sky + (i - nets.ap_bytes);
    *reinterpret_cast<uint32_t*>(sw + i) = *reinterpret_cast<const uint32_t*>(src);
  }
  __syncthreads();
  const unsigned char* w_ap = sw;
  const unsigned char* w_sky = sw + nets.ap_bytes;

  int x, y;
  const bool inside = tile_pixel(L, x, y);
  const int cx = inside ? x : 0, cy = inside ? y : 0;
  const size_t e = pix_offset(L, cx, cy);
  const size_t o = e * L.channels;
  const Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
  const PixelRay pr = pixel_ray(L, A, cx, cy);
  const f3 ray = pr.ray;
  const bool surface = inside && sid[e] >= 0;
  const float deg = 0.0174532925f;
  const float hz_cam = sky_horizon_zenith(A.cam_alt, A.bottom);
  const bool near_limb = fabsf(acosf(clampf(ray.y, -1.0f, 1.0f)) - hz_cam) < 0.5f * deg;

  // ---- surface pixels: features of the shell-clipped camera-to-surface segment
  float start = 0.0f, end = 0.0f;
  bool seg_ok = false, use_ap = false;
  float fx[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (surface && nets.ap != nullptr) {
    seg_ok = surface_interval(P, A.cam_alt, ray.y, A.bottom, norm(ld3(pos + o)), start, end);
    if (seg_ok) {
      const float o_y = A.bottom + A.cam_alt;
      const float hs = altitude_on_ray(A.cam_alt, ray.y, start, A.bottom);
      const f3 ps = mk(ray.x * start, o_y + ray.y * start, ray.z * start);
      const f3 up = ps * (1.0f / mx(norm(ps), 1.0f));
      const float mu_v = dot(ray, up), mu_s = dot(F.sun, up);
      const f3 tv = ray - up * mu_v, ts = F.sun - up * mu_s;
      const float nv = norm(tv), ns = norm(ts);
      const float cphi = (nv > 1e-6f && ns > 1e-6f) ? dot(tv, ts) / (nv * ns) : 1.0f;
      // twilight gate: the sun within 0.1 of the local horizon at either end or the middle
      float mu_far = 1.0f;
      for (int k = 1; k <= 2; ++k) {
        const float t = start + (end - start) * 0.5f * float(k);
        const f3 pt = mk(ray.x * t, o_y + ray.y * t, ray.z * t);
        mu_far = mn(mu_far, fabsf(dot(F.sun, pt) / mx(norm(pt), 1.0f)));
      }
      const bool twilight = fabsf(mu_s) < 0.1f || mu_far < 0.1f;
      use_ap = !twilight && !near_limb;
      geometry_features(P, A.bottom, hs, mu_v, mu_s, cphi, fx);
      fx[4] = nets.lhr_n;
      fx[5] = nets.lhm_n;
      fx[6] = 2.0f * logf(clampf(end - start, 1.0f, kSurrogateMaxLength)) / logf(kSurrogateMaxLength) - 1.0f;
    }
  }
  // ---- sky pixels: features of the camera's ray (cameras inside the shell)
  bool use_sky = false;
  float fs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (inside && !surface && nets.sky != nullptr && A.cam_alt <= P.top) {
    const float mu_s = F.sun.y;
    const float vl = sqrtf(ray.x * ray.x + ray.z * ray.z), sl = sqrtf(F.sun.x * F.sun.x + F.sun.z * F.sun.z);
    const float cphi = (vl > 1e-6f && sl > 1e-6f) ? (ray.x * F.sun.x + ray.z * F.sun.z) / (vl * sl) : 1.0f;
    use_sky = fabsf(mu_s) >= 0.1f && !near_limb;
    geometry_features(P, A.bottom, A.cam_alt, ray.y, mu_s, cphi, fs);
    fs[4] = nets.lhr_n;
    fs[5] = nets.lhm_n;
  }

  float yap[8] = {0, 0, 0, 0, 0, 0, 0, 0}, ysky[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (__any_sync(kAll, use_ap)) warp_mlp<4>(w_ap, mlp_bf16_layer_row(7), fx, yap);
  if (__any_sync(kAll, use_sky)) warp_mlp<3>(w_sky, mlp_bf16_layer_row(6), fs, ysky);

  uint32_t samples = 0;
  float err = -1.0f;
  if (inside) {
    f3 color = ld3(scene + o);
    if (surface) {
      if (seg_ok) {
        const bool check = use_ap && check_pixel(x, y, seed, check_fraction);
        f3 Lm = splat(0.0f), Tm = splat(1.0f);
        if (use_ap) {
          Lm = vmax(mk((__expf(yap[0]) - kSurrogateFloor) * A.E[0], (__expf(yap[1]) - kSurrogateFloor) * A.E[1],
                       (__expf(yap[2]) - kSurrogateFloor) * A.E[2]),
                    0.0f);
          Tm = mk(__expf(-mx(yap[3], 0.0f)), __expf(-mx(yap[4], 0.0f)), __expf(-mx(yap[5], 0.0f)));
        }
        if (!use_ap || check) {
          const f3 Lp = integrate_surface(P, F, A.cam_alt, ray, start, end, samples);
          const f3 Tp = surface_segment_t(P, F, A.cam_alt, ray, start, end);
          if (check) {
            const f3 cm = Lm + color * Tm, cp = Lp + color * Tp;
            const f3 d = vmax(cm - cp, 0.0f) + vmax(cp - cm, 0.0f);
            err = mx(mx(d.x / mx(cp.x, 1e-12f), d.y / mx(cp.y, 1e-12f)), d.z / mx(cp.z, 1e-12f));
          }
          Lm = Lp;  // re-integrated and gated pixels keep the plain result
          Tm = Tp;
        }
        color = Lm + color * Tm;
      }
    } else if (use_sky) {
      const f3 sky = vmax(mk((__expf(ysky[0]) - kSurrogateFloor) * A.E[0],
                             (__expf(ysky[1]) - kSurrogateFloor) * A.E[1],
                             (__expf(ysky[2]) - kSurrogateFloor) * A.E[2]),
                          0.0f);
      color = composite_sky_with(P, F, A, sky, ray, color, ld3(space + o), float(L.height));
    } else {
      color = composite_sky(P, F, A, svlut, ray, color, ld3(space + o), float(L.height));
    }
    color = vmax(color, 0.0f);
    hdr[o + 0] = color.x;
    hdr[o + 1] = color.y;
    hdr[o + 2] = color.z;
  }
  warp_count(samples, counter);
  // error statistics of the re-integrated pixels: count, sum, max, gated surface pixels
  if (stats != nullptr) {
    const bool checked = err >= 0.0f;
    const unsigned gated = __ballot_sync(kAll, surface && seg_ok && !use_ap);
    float s = checked ? err : 0.0f, m = checked ? err : 0.0f;
#pragma unroll
    for (int k = 16; k > 0; k >>= 1) {
      s += __shfl_xor_sync(kAll, s, k);
      m = mx(m, __shfl_xor_sync(kAll, m, k));
    }
    const unsigned n_checked = __popc(__ballot_sync(kAll, checked));
    if ((threadIdx.x & 31) == 0) {
      if (n_checked) {
        atomicAdd(stats + 0, float(n_checked));
        atomicAdd(stats + 1, s);
        atomicMax(reinterpret_cast<int*>(stats + 2), __float_as_int(m));
      }
      if (gated) atomicAdd(stats + 3, float(__popc(gated)));
    }
  }
}

}  // namespace

cudaError_t launch_gen_samples(const SurrogateSetDev* sets, int n_sets, int kind, long long n, unsigned long long seed,
                               const float E[3], float ar, float* features, float* targets,
                               unsigned long long* counter, cudaStream_t s) {
  const f3 e3 = {E[0], E[1], E[2]};
  k_gen_samples<<<unsigned((n + 127) / 128), 128, 0, s>>>(sets, n_sets, kind, n, seed, e3, ar,
                                                         features, targets, counter);
  return cudaGetLastError();
}

cudaError_t launch_composite_surrogate(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                                       const float* scene, const float* space, const int32_t* sid, const float* pos,
                                       const float4* tlut, const float4* mslut, const float4* svlut,
                                       const SurrogateNets& nets, unsigned seed, float check_fraction, float* hdr,
                                       float* stats, unsigned long long* counter, cudaStream_t s) {
  const int smem = nets.ap_bytes + nets.sky_bytes;
  cudaError_t e = cudaFuncSetAttribute(k_composite_surrogate, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const dim3 grid((L.width + 15) / 16, (L.height + 15) / 16);
  k_composite_surrogate<<<grid, 256, smem, s>>>(P, L, A, scene, space, sid, pos, tlut, mslut, svlut, nets, seed,
                                                check_fraction, hdr, stats, counter);
  return cudaGetLastError();
}

}  // namespace atm
