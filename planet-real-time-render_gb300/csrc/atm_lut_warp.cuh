// atm_lut_warp.cuh - warp-cooperative evaluation of one sky-view texel and
// one aerial-perspective column (reference atmosphere/renderer.py
// :1208-1302 and :1304-1420).  Shared by the single-LUT kernels and the
// persistent batched builder; every lane of the calling warp must call.
#pragma once

#include "atm_device.cuh"

namespace atm {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ f3 shfl_xor3(f3 v, int m) {
  return {__shfl_xor_sync(kFull, v.x, m), __shfl_xor_sync(kFull, v.y, m), __shfl_xor_sync(kFull, v.z, m)};
}
__device__ __forceinline__ Seg shfl_down_seg(Seg s, int o) {
  return {{__shfl_down_sync(kFull, s.L.x, o), __shfl_down_sync(kFull, s.L.y, o), __shfl_down_sync(kFull, s.L.z, o)},
          {__shfl_down_sync(kFull, s.T.x, o), __shfl_down_sync(kFull, s.T.y, o), __shfl_down_sync(kFull, s.T.z, o)}};
}
__device__ __forceinline__ Seg shfl_up_seg(Seg s, int o) {
  return {{__shfl_up_sync(kFull, s.L.x, o), __shfl_up_sync(kFull, s.L.y, o), __shfl_up_sync(kFull, s.L.z, o)},
          {__shfl_up_sync(kFull, s.T.x, o), __shfl_up_sync(kFull, s.T.y, o), __shfl_up_sync(kFull, s.T.z, o)}};
}
__device__ __forceinline__ Seg seg_identity() { return {splat(0.0f), splat(1.0f)}; }

// Ordered reduction of 32 consecutive segments; lane 0 receives the total.
__device__ __forceinline__ Seg warp_compose(Seg s) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    Seg other = shfl_down_seg(s, o);
    if ((threadIdx.x & 31) + o < 32) s = seg_then(s, other);
  }
  return s;
}
// Ordered inclusive scan: lane i receives segment 0 then ... then i.
__device__ __forceinline__ Seg warp_scan(Seg s) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    Seg before = shfl_up_seg(s, o);
    if (lane >= o) s = seg_then(before, s);
  }
  return s;
}


// One sky-view texel (x, y): lanes split the march steps, the per-step
// (L, T) segments are composed in ray order; lane 0 stores the texel.
// Returns the radiance samples this lane evaluated.
__device__ __forceinline__ uint32_t sky_view_texel(const DevParams& P, const Frame& F, float cam_alt, int x, int y,
                                                   float4* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const float bottom = F.bottom;
  const float sh = mx(cam_alt, 0.0f);
  float az = (float(x) + 0.5f) / float(P.sv_w) * kPiF;
  float vv = (float(y) + 0.5f) / float(P.sv_h);
  float zen = sky_v_to_zenith(vv, sky_horizon_zenith(sh, bottom));
  float vs, vc, saz, caz;
  sincosf(zen, &vs, &vc);
  if (far_camera(P, bottom, sh)) {
    // seen from many planet radii the whole planet spans a few degrees
    // around the nadir: the same mapping in nadir angles keeps the digits
    // that zen itself, near pi, loses.  The horizon's nadir angle
    // pi - hz = acos(rho / r) = asin(R / r): acos of rho / r ~ 1 amplifies one
    // float ulp of its argument to ~2e-6 rad (and 1e-7 rad of direction
    // moves a limb texel's radiance by 0.2%); asin of R / r is well conditioned
    const float nh = asinf(clampf(__fdiv_rn(bottom, bottom + sh), 0.0f, 1.0f));
    float nadir;
    if (vv >= 0.5f) {
      const float local = 2.0f * vv - 1.0f;
      nadir = nh * (1.0f - local * local);  // pi - (hz + (pi - hz) local^2)
    } else {
      const float inv = 1.0f - 2.0f * vv;
      nadir = nh + (kPiF - nh) * (inv * inv);  // pi - hz (1 - inv^2)
    }
    sincosf(nadir, &vs, &vc);
    vc = -vc;
  }
  sincosf(az, &saz, &caz);
  f3 ray = mk(vs * caz, vc, vs * saz);
  const RayGeom G = ray_geom(P, bottom, sh, vc, vs);
  float start, end;
  bool valid, ground;
  segment_of(P, G, bottom, start, end, valid, ground);
  Seg acc = seg_identity();
  uint32_t samples = 0;
  if (valid) {
    const RaySource rs = make_ray_source(P, F, G, ray);
    const RayWarp rw = make_warp(G.tc, start, end);
    const int n = P.sv_steps;
    const int per = (n + 31) >> 5;
    const int i0 = lane * per;
    const int i1 = min(i0 + per, n);
    if (i0 < i1) {
      float d0 = warp_at(rw, float(i0) / float(n));
      for (int i = i0; i < i1; ++i) {
        float d1 = warp_at(rw, float(i + 1) / float(n));
        float vis;
        acc = seg_then(acc, source_segment<true>(P, F, rs, d0, d1, vis));
        d0 = d1;
      }
      samples = uint32_t(i1 - i0);
    }
  }
  acc = warp_compose(acc);
  if (lane == 0) out[y * P.sv_w + x] = to4(vmax(acc.L, 0.0f));
  return samples;
}

// Segment of depth slice k along a column's prefix interval [as, ae].
__device__ __forceinline__ Seg aerial_slice(const DevParams& P, const Frame& F, const RaySource& rs, float as,
                                            float ae, bool valid, int k, float closest_raw, uint32_t& samples) {
  Seg acc = seg_identity();
  const float denom = float(P.ap_d - 1);
  float prev = k == 0 ? as : as + (ae - as) * (float(k - 1) / denom);
  float target = as + (ae - as) * (float(k) / denom);
  if (valid) {
    float is = mx(prev, as);
    float ie = mn(target, ae);
    if (ie > is) {
      const int n = P.ap_steps;
      const RayWarp rw = make_warp(closest_raw, is, ie);
      float d0 = warp_at(rw, 0.0f);
      for (int s = 0; s < n; ++s) {
        float d1 = warp_at(rw, float(s + 1) / float(n));
        float vis;
        acc = seg_then(acc, source_segment<true>(P, F, rs, d0, d1, vis));
        d0 = d1;
      }
      samples += uint32_t(n);
    }
  }
  return acc;
}

// Camera of an aerial-perspective volume.
struct AerialView {
  float aspect, cam_alt;
  f3 right, up, fwd;
  float tanfov;
};

// One froxel column (x, y): lanes take depth slices, an ordered inclusive
// scan gives every slice its cumulative in-scattering.  Returns the samples
// this lane evaluated (the second pass of deep volumes is not counted).
__device__ __forceinline__ uint32_t aerial_column(const DevParams& P, const Frame& F, const AerialView& V, int x,
                                                  int y, float4* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const float bottom = F.bottom;
  float u = (float(x) + 0.5f) / float(P.ap_w);
  float v = (float(y) + 0.5f) / float(P.ap_h);
  float sx = (u * 2.0f - 1.0f) * V.aspect;
  float sy = v * 2.0f - 1.0f;
  f3 rv = (V.right * sx + V.up * sy) + V.fwd / V.tanfov;
  f3 ray = rv * (1.0f / norm(rv));
  float as, ae;
  bool valid;
  const RayGeom G = ray_geom(P, bottom, V.cam_alt, ray.y, sqrtf(ray.x * ray.x + ray.z * ray.z));
  aerial_prefix_of(P, G, bottom, as, ae, valid);
  const RaySource rs = make_ray_source(P, F, G, ray);
  const float closest_raw = G.tc;
  const int depth = P.ap_d;
  const int per = (depth + 31) >> 5;
  const size_t plane = size_t(P.ap_w) * P.ap_h;
  Seg run = seg_identity();
  uint32_t samples = 0;
  for (int k = lane * per; k < min(lane * per + per, depth); ++k)
    run = seg_then(run, aerial_slice(P, F, rs, as, ae, valid, k, closest_raw, samples));
  Seg incl = warp_scan(run);
  Seg prefix = shfl_up_seg(incl, 1);
  if (lane == 0) prefix = seg_identity();
  if (per == 1) {
    if (lane < depth) out[size_t(lane) * plane + size_t(y) * P.ap_w + x] = to4(vmax(incl.L, 0.0f));
    return samples;
  }
  Seg acc = prefix;
  uint32_t recomputed = 0;
  for (int k = lane * per; k < min(lane * per + per, depth); ++k) {
    acc = seg_then(acc, aerial_slice(P, F, rs, as, ae, valid, k, closest_raw, recomputed));
    out[size_t(k) * plane + size_t(y) * P.ap_w + x] = to4(vmax(acc.L, 0.0f));
  }
  return samples;
}

}  // namespace atm
