// atm_luts.cu - Transmittance, Multi-scattering, Sky-view and Aerial-perspective
// LUT builds (reference atmosphere/renderer.py :1034-1420) for sm_103a.
//
// Work decomposition (the reference runs one Taichi thread per texel, each
// marching its ray sequentially):
//  - transmittance: 8 lanes per texel split the 40 optical-depth steps and
//    sum with xor shuffles;
//  - multi-scattering: one thread per (texel, direction); a block holds one
//    texel; the direction sums are added in the reference's order;
//  - sky-view: one warp per texel, lanes over march steps; the per-step
//    (radiance, transmittance) segments are composed in ray order by a
//    shuffle tree ((L1,T1) then (L2,T2) = (L1 + T1 L2, T1 T2));
//  - aerial perspective: one warp per froxel column, lanes over depth
//    slices; an ordered inclusive shuffle scan of the slice segments gives
//    each slice's cumulative in-scattering.
// Every LUT is float4 row-major [z][y][x]: stores are 16-byte and coalesced
// along x.
#include <cuda_runtime.h>

#include <algorithm>

#include "atm_device.cuh"
#include "atm_kernels.h"
#include "atm_lut_warp.cuh"

namespace atm {
namespace {

// ---- transmittance (:1034-1063, :570-607) ----------------------------------
constexpr int kTLanes = 8;

__global__ void __launch_bounds__(256) k_transmittance(DevParams P, float bottom, float4* __restrict__ out) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int texel = gid / kTLanes;
  const int sub = gid % kTLanes;
  const int n_texels = P.t_w * P.t_h;
  const bool active = texel < n_texels;
  const int t = active ? texel : 0;
  const int x = t % P.t_w, y = t / P.t_w;
  float u = (float(x) + 0.5f) / float(P.t_w);
  float v = (float(y) + 0.5f) / float(P.t_h);
  float h, c, dist;
  t_uv_to_ray(P, u, v, bottom, h, c, dist);
  float s = sqrtf(mx(1.0f - c * c, 0.0f));
  float radius = bottom + h;
  f3 o = mk(0.0f, radius, 0.0f);
  f3 ray = mk(s, c, 0.0f);
  float closest_raw = -dot(o, ray);
  f3 od = splat(0.0f);
  const int n = P.t_steps;
  for (int i = sub; i < n; i += kTLanes) {
    float d0 = warp_boundary(closest_raw, 0.0f, dist, float(i) / float(n));
    float d1 = warp_boundary(closest_raw, 0.0f, dist, float(i + 1) / float(n));
    float step = d1 - d0;
    float mid = (d0 + d1) * 0.5f;
    float alt = norm(o + ray * mid) - bottom;
    od = od + extinction_of(P, density(P, alt)) * step;
  }
#pragma unroll
  for (int m = 1; m < kTLanes; m <<= 1) od = od + shfl_xor3(od, m);
  if (active && sub == 0) out[y * P.t_w + x] = to4(vclamp(vexp(-vmin(od, 80.0f)), 0.0f, 1.0f));
}

// ---- multi-scattering (:1065-1206) ------------------------------------------
constexpr int kMaxDirs = 128;

__global__ void __launch_bounds__(kMaxDirs) k_multi_scattering(DevParams P, float bottom, f3 E, float ar,
                                                               const float4* __restrict__ tlut,
                                                               float4* __restrict__ out,
                                                               unsigned long long* counter) {
  __shared__ f3 s_l[kMaxDirs];
  __shared__ f3 s_f[kMaxDirs];
  const int texel = blockIdx.x;
  const int x = texel % P.ms_w, y = texel / P.ms_w;
  const int di = threadIdx.x;
  float u = (float(x) + 0.5f) / float(P.ms_w);
  float v = (float(y) + 0.5f) / float(P.ms_h);
  float h0 = v * v * P.top;
  float radius = bottom + h0;
  float sc = sun_u_to_cosine(u, h0, bottom);
  float ss = sqrtf(mx(1.0f - sc * sc, 0.0f));
  Frame F = make_frame(P, tlut, nullptr, bottom, ar, mk(ss, sc, 0.0f), E);
  f3 o = mk(0.0f, radius, 0.0f);
  f3 dL = splat(0.0f), dF = splat(0.0f);
  uint32_t samples = 0;
  if (di < P.ms_dirs) {
    const int ndir = P.ms_dirs;
    float si = float(di) + 0.5f;
    float dc = 1.0f - 2.0f * si / float(ndir);
    float ds = sqrtf(mx(1.0f - dc * dc, 0.0f));
    float az = float(di) * 2.39996323f;
    float saz, caz;
    sincosf(az, &saz, &caz);
    f3 ray = mk(ds * caz, dc, ds * saz);
    float start, end;
    bool valid, ground;
    segment_vec(P, o, ray, bottom, start, end, valid, ground);
    if (valid) {
      const float phase_r = rayleigh_phase(P, clampf(dot(ray, F.sun), -1.0f, 1.0f));
      const float phase_m = mie_phase(P, clampf(dot(ray, F.sun), -1.0f, 1.0f));
      const float closest_raw = -dot(o, ray);
      f3 pT = splat(1.0f);
      const int n = P.ms_steps;
      float d0 = warp_boundary(closest_raw, start, end, 0.0f);
      for (int pi = 0; pi < n; ++pi) {
        float d1 = warp_boundary(closest_raw, start, end, float(pi + 1) / float(n));
        float dist = (d0 + d1) * 0.5f;
        float step = d1 - d0;
        f3 point = o + ray * dist;
        float hh = altitude_on_ray(h0, dc, dist, bottom);
        Density d = density(P, hh);
        f3 sT, sI;
        segment_integral(extinction_of(P, d), step, sT, sI);
        float rr = norm(point);
        f3 radial = point / mx(rr, 1.0f);
        float psc = dot(radial, F.sun);
        float vis;
        f3 st = sample_solar_t(P, F, hh, psc, horizon_at(hh, bottom), vis);
        f3 src = (F.E * st) * (arr3(P.beta_r) * d.r * phase_r + arr3(P.beta_ms) * d.m * phase_m);
        dL = dL + pT * src * sI;
        dF = dF + pT * scattering_of(P, d) * sI;
        pT = pT * sT;
        d0 = d1;
      }
      samples = uint32_t(n);
      if (ground) {
        f3 gp = o + ray * end;
        f3 gn = gp * (1.0f / norm(gp));  // Taichi normalized(): v * (1/|v|)
        float gsc = dot(gn, F.sun);
        float vis;
        f3 gT = sample_solar_t(P, F, 0.0f, gsc, horizon_at(0.0f, bottom), vis);
        f3 gL = arr3(P.albedo) * F.E * gT * mx(gsc, 0.0f) / kPiF;
        dL = dL + pT * gL;
      }
    }
  }
  warp_count(samples, counter);
  s_l[di] = dL;
  s_f[di] = dF;
  __syncthreads();
  if (di == 0) {
    f3 lsum = splat(0.0f), fsum = splat(0.0f);
    for (int k = 0; k < P.ms_dirs; ++k) {
      lsum = lsum + s_l[k];
      fsum = fsum + s_f[k];
    }
    f3 avg_l = lsum / float(P.ms_dirs);
    f3 avg_f = vclamp(fsum / float(P.ms_dirs), 0.0f, 0.95f);
    out[y * P.ms_w + x] = to4(vmax(avg_l / (splat(1.0f) - avg_f), 0.0f));
  }
}

// ---- sky-view (:1208-1302) and aerial perspective (:1304-1420) -----------------
__global__ void __launch_bounds__(256) k_sky_view(DevParams P, float bottom, float cam_alt, float sun_cos, f3 E,
                                                  float ar, const float4* __restrict__ tlut,
                                                  const float4* __restrict__ mslut, float4* __restrict__ out,
                                                  unsigned long long* counter) {
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp_id >= P.sv_w * P.sv_h) return;  // warp-uniform
  float ss = sqrtf(mx(1.0f - sun_cos * sun_cos, 0.0f));
  Frame F = make_frame(P, tlut, mslut, bottom, ar, mk(ss, sun_cos, 0.0f), E);
  uint32_t samples = sky_view_texel(P, F, cam_alt, warp_id % P.sv_w, warp_id / P.sv_w, out);
  warp_count(samples, counter);
}

__global__ void __launch_bounds__(256) k_aerial(DevParams P, float aspect, float bottom, float cam_alt, f3 sun, f3 E,
                                                float ar, f3 right, f3 up, f3 fwd, float tanfov,
                                                const float4* __restrict__ tlut, const float4* __restrict__ mslut,
                                                float4* __restrict__ out, unsigned long long* counter) {
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp_id >= P.ap_w * P.ap_h) return;  // warp-uniform
  Frame F = make_frame(P, tlut, mslut, bottom, ar, sun, E);
  AerialView V{aspect, cam_alt, right, up, fwd, tanfov};
  uint32_t samples = aerial_column(P, F, V, warp_id % P.ap_w, warp_id / P.ap_w, out);
  warp_count(samples, counter);
}

__global__ void k_lut_to_fields(const float4* __restrict__ lut, int w, int h, int d, float* __restrict__ dst) {
  const size_t n = size_t(w) * h * d;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    // dst index (x, y, z) in (W, H, D) order
    size_t z = i % d, y = (i / d) % h, x = i / (size_t(d) * h);
    float4 v = lut[(z * h + y) * w + x];
    dst[i * 3 + 0] = v.x;
    dst[i * 3 + 1] = v.y;
    dst[i * 3 + 2] = v.z;
  }
}

__global__ void k_fields_to_lut(const float* __restrict__ src, int w, int h, int d, float4* __restrict__ lut) {
  const size_t n = size_t(w) * h * d;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    size_t z = i % d, y = (i / d) % h, x = i / (size_t(d) * h);
    lut[(z * h + y) * w + x] = make_float4(src[i * 3 + 0], src[i * 3 + 1], src[i * 3 + 2], 0.0f);
  }
}

inline f3 host3(const float* v) { return {v[0], v[1], v[2]}; }

}  // namespace

cudaError_t launch_transmittance(const DevParams& P, float bottom, float4* out, cudaStream_t s) {
  const int threads = 256;
  const int total = P.t_w * P.t_h * kTLanes;
  k_transmittance<<<(total + threads - 1) / threads, threads, 0, s>>>(P, bottom, out);
  return cudaGetLastError();
}

cudaError_t launch_multi_scattering(const DevParams& P, float bottom, const float E[3], float ar,
                                    const float4* tlut, float4* out, unsigned long long* counter, cudaStream_t s) {
  if (P.ms_dirs > kMaxDirs) return cudaErrorInvalidValue;
  const int threads = ((P.ms_dirs + 31) / 32) * 32;
  k_multi_scattering<<<P.ms_w * P.ms_h, threads, 0, s>>>(P, bottom, host3(E), ar, tlut, out, counter);
  return cudaGetLastError();
}

cudaError_t launch_sky_view(const DevParams& P, float bottom, float cam_alt, float sun_cos, const float E[3],
                            float ar, const float4* tlut, const float4* mslut, float4* out,
                            unsigned long long* counter, cudaStream_t s) {
  const int threads = 256;
  const long long total = 32LL * P.sv_w * P.sv_h;
  k_sky_view<<<unsigned((total + threads - 1) / threads), threads, 0, s>>>(P, bottom, cam_alt, sun_cos, host3(E), ar,
                                                                          tlut, mslut, out, counter);
  return cudaGetLastError();
}

cudaError_t launch_aerial(const DevParams& P, int width, int height, float bottom, float cam_alt, const float sun[3],
                          const float E[3], float ar, const float right[3], const float up[3], const float fwd[3],
                          float tanfov, const float4* tlut, const float4* mslut, float4* out,
                          unsigned long long* counter, cudaStream_t s) {
  const int threads = 256;
  const long long total = 32LL * P.ap_w * P.ap_h;
  const float aspect = float(width) / float(height);
  k_aerial<<<unsigned((total + threads - 1) / threads), threads, 0, s>>>(
      P, aspect, bottom, cam_alt, host3(sun), host3(E), ar, host3(right), host3(up), host3(fwd), tanfov, tlut, mslut,
      out, counter);
  return cudaGetLastError();
}

cudaError_t launch_lut_to_fields(const float4* lut, int w, int h, int d, float* dst, cudaStream_t s) {
  const size_t n = size_t(w) * h * d;
  const int threads = 256;
  const unsigned blocks = unsigned(std::min<size_t>((n + threads - 1) / threads, 4096));
  k_lut_to_fields<<<blocks, threads, 0, s>>>(lut, w, h, d, dst);
  return cudaGetLastError();
}

cudaError_t launch_fields_to_lut(const float* src, int w, int h, int d, float4* lut, cudaStream_t s) {
  const size_t n = size_t(w) * h * d;
  const int threads = 256;
  const unsigned blocks = unsigned(std::min<size_t>((n + threads - 1) / threads, 4096));
  k_fields_to_lut<<<blocks, threads, 0, s>>>(src, w, h, d, lut);
  return cudaGetLastError();
}

}  // namespace atm
