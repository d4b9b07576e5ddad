// atm_surrogate.cu - learned surrogates of the sky radiance and of the
// camera-to-surface in-scattering / transmittance.
//
//  * k_gen_samples: training samples produced by the plain integrator itself
//    (the same device functions as the LUT builds and the composite).
//  * k_composite_surrogate + k_surrogate_fallback: the COMPOSITE view with
//    the per-pixel limb integrator (renderer.py :1667-1786) replaced by a
//    BF16 tensor-core MLP and the sky-view lookup (:1474-1525) by a second
//    one.  Pixels where a gate trips (view ray within 0.5 deg of the limb,
//    sun within 0.1 of the local horizon) and a random fraction of the MLP
//    pixels (the error check) go to a queue; the second kernel runs the plain
//    integrator over the queue densely, so a few plain pixels do not stall
//    whole warps of MLP pixels.
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
#include "atm_mlp_tc.cuh"

namespace atm {

namespace {

constexpr unsigned kAll = 0xffffffffu;

// x[0..3]: altitude, view, sun, relative azimuth at the segment's first point.
__device__ __forceinline__ void geometry_features(const DevParams& P, float bottom, float h, float mu_v, float mu_s,
                                                  float cos_dphi, float* x) {
  const float hn = clampf(h * P.inv_top, 0.0f, 1.0f);
  x[0] = 2.0f * sqrtf(hn) - 1.0f;
  x[1] = 2.0f * sky_zenith_to_v(acosf(clampf(mu_v, -1.0f, 1.0f)), sky_horizon_zenith(h, bottom)) - 1.0f;
  x[2] = 2.0f * sun_cosine_to_u(clampf(mu_s, -1.0f, 1.0f), horizon_cosine(h, bottom)) - 1.0f;
  x[3] = clampf(cos_dphi, -1.0f, 1.0f);
}

// Sun (multi-scattering u mapping) and altitude features, x[0] and x[1], of
// the point at distance t along a ray leaving (0, o_y, 0) (G: its geometry).
// Where a segment's light comes from depends on where it ends and how low it
// dips as much as on where it starts: with these points given, the sky
// network's held-out error drops by a quarter and the aerial network's on
// camera-to-surface segments to a third.  Returns the point's sun cosine.
__device__ __forceinline__ float point_features(const DevParams& P, float bottom, const RayGeom& G, f3 ray, float o_y,
                                                f3 sun, float t, float* x) {
  const f3 pt = mk(ray.x * t, o_y + ray.y * t, ray.z * t);
  const float mu = clampf(dot(sun, pt) / mx(norm(pt), 1.0f), -1.0f, 1.0f);
  const float h = altitude_at(G, t, bottom);
  x[0] = 2.0f * sun_cosine_to_u(mu, horizon_cosine(h, bottom)) - 1.0f;
  x[1] = 2.0f * sqrtf(clampf(h * P.inv_top, 0.0f, 1.0f)) - 1.0f;
  return mu;
}
// Aerial x[7..10]: the segment's end, then its middle.  Returns the smaller
// |sun cosine| of the two (the twilight gate); `mu_end`, `mu_mid` receive
// the cosines themselves.
__device__ __forceinline__ float segment_features(const DevParams& P, float bottom, const RayGeom& G, f3 ray,
                                                  float o_y, f3 sun, float start, float end, float* x,
                                                  float& mu_end, float& mu_mid) {
  mu_end = point_features(P, bottom, G, ray, o_y, sun, end, x + 7);
  mu_mid = point_features(P, bottom, G, ray, o_y, sun, 0.5f * (start + end), x + 9);
  return mn(fabsf(mu_end), fabsf(mu_mid));
}
// Sky x[6..9]: the end of the ray's march (the shell top or the ground),
// then its lowest point (the closest approach, clamped to the march).
__device__ __forceinline__ void sky_ray_features(const DevParams& P, float bottom, float h, f3 ray, f3 sun, float* x) {
  const RayGeom G = camera_ray_geom(P, bottom, h, ray);
  float start, end;
  bool valid, ground;
  segment_of(P, G, bottom, start, end, valid, ground);
  if (!valid) start = end = 0.0f;
  const float o_y = bottom + mx(h, 0.0f);
  point_features(P, bottom, G, ray, o_y, sun, end, x + 6);
  point_features(P, bottom, G, ray, o_y, sun, clampf(G.tc, start, end), x + 8);
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
  const RayGeom G = camera_ray_geom(P, F.bottom, h, ray);
  segment_of(P, G, F.bottom, start, end, valid, ground);
  Seg acc = {splat(0.0f), splat(1.0f)};
  if (valid) {
    const RaySource rs = make_ray_source(P, F, G, ray);
    const RayWarp rw = make_warp(G.tc, start, end);
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

// Aerial samples may be shaped toward camera-to-surface segments: a share
// starts at the shell top (feature 0 = 1; every segment seen from above the
// shell starts there) and a share ends at a surface altitude, where the ray
// reaches it (the segment's length then follows from the geometry).
__global__ void __launch_bounds__(128) k_gen_samples(const SurrogateSetDev* __restrict__ sets, int n_sets, int kind,
                                                     long long n, unsigned long long seed, SampleShaping shaping,
                                                     f3 E, float ar, float* __restrict__ features,
                                                     float* __restrict__ targets,
                                                     unsigned long long* __restrict__ counter) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  uint32_t samples = 0;
  if (i < n) {
    const SurrogateSetDev& S = sets[min(int(uniform01(seed, i, 0) * n_sets), n_sets - 1)];
    const DevParams& P = S.P;
    const float R = S.bottom;
    float x[16];
    for (int k = 0; k < 4; ++k) x[k] = 2.0f * uniform01(seed, i, k + 1) - 1.0f;
    if (shaping.x0_lo < shaping.x0_hi) x[0] = shaping.x0_lo + (shaping.x0_hi - shaping.x0_lo) * uniform01(seed, i, 9);
    if (kind == 1 && uniform01(seed, i, 6) < shaping.top_fraction) x[0] = 1.0f;
    // invert the feature maps
    const float h = P.top * 0.25f * (x[0] + 1.0f) * (x[0] + 1.0f);
    const float zen = sky_v_to_zenith(0.5f * (x[1] + 1.0f), sky_horizon_zenith(h, R));
    float sv, mu_v;
    sincosf(zen, &sv, &mu_v);
    // the sun: uniform in the feature, or for a share uniform in zenith angle
    // (the feature's horizon-concentrating map leaves a high sun sparse)
    const float mu_s = uniform01(seed, i, 10) < shaping.sun_angle_fraction
                           ? cosf(shaping.sun_angle_max * uniform01(seed, i, 11))
                           : sun_u_to_cosine(0.5f * (x[2] + 1.0f), h, R);
    const float ss = sqrtf(mx(1.0f - mu_s * mu_s, 0.0f));
    const float cphi = x[3], sphi = sqrtf(mx(1.0f - cphi * cphi, 0.0f));
    const f3 ray = mk(sv, mu_v, 0.0f);
    const f3 sun = mk(ss * cphi, mu_s, ss * sphi);
    geometry_features(P, R, h, mu_v, mu_s, cphi, x);  // rounding-consistent features
    x[4] = S.lhr_n;
    x[5] = S.lhm_n;
    const Frame F = make_frame(P, S.tlut, S.mslut, R, ar, sun, E);
    const f3 inv_e = mk(1.0f / E.x, 1.0f / E.y, 1.0f / E.z);
    if (kind == 0) {  // sky: 10 features -> log(L/E + floor)
      const f3 L = sky_radiance(P, F, h, ray) * inv_e;
      samples = uint32_t(P.sv_steps);
      sky_ray_features(P, R, h, ray, sun, x);
      for (int k = 0; k < kSurrogateSkyIn; ++k) features[i * kSurrogateSkyIn + k] = x[k];
      targets[i * 3 + 0] = logf(L.x + kSurrogateFloor);
      targets[i * 3 + 1] = logf(L.y + kSurrogateFloor);
      targets[i * 3 + 2] = logf(L.z + kSurrogateFloor);
    } else {  // aerial: + log length -> log(L/E + floor), optical depth
      const float u = uniform01(seed, i, 5);
      float len = expf(u * logf(kSurrogateMaxLength));
      x[6] = 2.0f * u - 1.0f;
      if (uniform01(seed, i, 7) < shaping.surface_fraction) {
        const float he = shaping.surface_min + (shaping.surface_max - shaping.surface_min) * uniform01(seed, i, 8);
        float nr, fr;
        bool hit;
        shell_roots(h, mu_v, he, R, nr, fr, hit);
        const float t = nr > 0.0f ? nr : fr;
        if (hit && t >= 1.0f && t <= kSurrogateMaxLength) {
          len = t;
          x[6] = 2.0f * logf(len) / logf(kSurrogateMaxLength) - 1.0f;
        }
      }
      f3 L = splat(0.0f), T = splat(1.0f);
      float start, end;
      const RayGeom G = ray_geom(P, R, h, mu_v, sv);
      if (surface_interval(P, G, R, len, start, end)) {
        L = integrate_surface(P, F, G, ray, start, end, samples) * inv_e;
        T = surface_segment_t(P, F, G, ray, start, end);
      } else {
        start = end = 0.0f;
      }
      float mu_end, mu_mid;
      segment_features(P, R, G, ray, R + h, sun, start, end, x, mu_end, mu_mid);
      for (int k = 0; k < kSurrogateApIn; ++k) features[i * kSurrogateApIn + k] = x[k];
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

__device__ __forceinline__ bool check_pixel(int x, int y, unsigned seed, float fraction) {
  unsigned h = (unsigned(x) * 0x8DA6B343u) ^ (unsigned(y) * 0xD8163841u) ^ (seed * 0x9E3779B1u);
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  return float(h >> 8) * (1.0f / 16777216.0f) < fraction;
}

// A pixel's index in storage order (the image's contiguous axis first), the
// order of the calibration scratch image.
__device__ __forceinline__ size_t storage_index(const ImageLayout& L, int x, int y) {
  return L.sy <= L.sx ? size_t(x) * size_t(L.height) + size_t(y) : size_t(y) * size_t(L.width) + size_t(x);
}

// Largest per-channel error of `got` relative to `ref` (floor 1e-6 E).
__device__ __forceinline__ float color_error(f3 got, f3 ref, f3 E) {
  const f3 d = vmax(got - ref, 0.0f) + vmax(ref - got, 0.0f);
  return mx(mx(d.x / mx(ref.x, 1e-6f * E.x), d.y / mx(ref.y, 1e-6f * E.y)), d.z / mx(ref.z, 1e-6f * E.z));
}

// Radiance of a network's log output ln(L / E + floor), per channel.
__device__ __forceinline__ f3 net_radiance(const float (&y)[8], const float* E, f3 floor) {
  return vmax(mk((__expf(y[0]) - floor.x) * E[0], (__expf(y[1]) - floor.y) * E[1], (__expf(y[2]) - floor.z) * E[2]),
              0.0f);
}

enum PixelKind : int { kNone = 0, kSurfMlp, kSurfPlain, kSurfEmpty, kSkyMlp, kSkyLut };

// 256 threads = two tiles of 128 pixels (warps 0-3, 4-7); a pixel is one
// tensor-memory lane of its tile.  Tensor memory (256 columns): tile t holds
// its accumulators at column 128 t and its activations at 128 t + 64.
constexpr uint32_t kSurrogateTmemCols = 256;

// kShade: the surface colour comes from the fused surface lighting and
// shading (shaded_scene) instead of the scene image.
template <bool kShade>
__global__ void __launch_bounds__(256, 3) k_composite_surrogate(
    DevParams P, ImageLayout L, CompositeScalars A, const float* __restrict__ scene, const float* __restrict__ space,
    const int32_t* __restrict__ sid, const float* __restrict__ pos, const float4* __restrict__ tlut,
    const float4* __restrict__ mslut, const float4* __restrict__ svlut, SurrogateNets nets, SurrogateQueue Q,
    float* __restrict__ hdr, ShadeParams S, ShadeImages I) {
  extern __shared__ __align__(128) unsigned char smem[];  // the aerial network, then the sky network
  __shared__ __align__(8) uint64_t s_mbar[3];  // the two tiles' MMA completions, the weights' arrival
  __shared__ uint32_t s_tmem;
  const int wbytes = nets.ap_bytes + nets.sky_bytes;
  if (threadIdx.x == 0) {
    tc::mbar_init(&s_mbar[0], 1);
    tc::mbar_init(&s_mbar[1], 1);
    tc::mbar_init(&s_mbar[2], 1);
    tc::mbar_init_fence();
  }
  __syncthreads();
  // the weights arrive by bulk copy while the block computes its features
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&s_mbar[2], uint32_t(wbytes));
    if (nets.ap_bytes > 0) tc::bulk_g2s(smem, nets.ap, uint32_t(nets.ap_bytes), &s_mbar[2]);
    if (nets.sky_bytes > 0) tc::bulk_g2s(smem + nets.ap_bytes, nets.sky, uint32_t(nets.sky_bytes), &s_mbar[2]);
  }
  const int tile = threadIdx.x >> 7;

  int x, y;
  const bool inside = tile_pixel(L, x, y);
  const int cx = inside ? x : 0, cy = inside ? y : 0;
  const size_t e = pix_offset(L, cx, cy);
  const size_t o = e * L.channels;
  const Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
  const f3 ray = pixel_ray(L, A, cx, cy).ray;
  const bool near_limb =
      fabsf(acosf(clampf(ray.y, -1.0f, 1.0f)) - sky_horizon_zenith(A.cam_alt, A.bottom)) < nets.limb_rad;

  int kind = kNone;
  float fx[16] = {};
  float start = 0.0f, end = 0.0f;
  if (inside) {
    if (sid[e] >= 0) {
      const RayGeom G = camera_ray_geom(P, A.bottom, A.cam_alt, ray);
      if (!surface_interval(P, G, A.bottom, norm(ld3(pos + o)), start, end)) {
        kind = kSurfEmpty;
      } else if (nets.ap == nullptr || near_limb) {
        kind = kSurfPlain;
      } else {
        // features at the segment's first point inside the shell
        const float o_y = A.bottom + A.cam_alt;
        const float hs = altitude_at(G, start, A.bottom);
        const f3 ps = mk(ray.x * start, o_y + ray.y * start, ray.z * start);
        const f3 up = ps * (1.0f / mx(norm(ps), 1.0f));
        const float mu_v = dot(ray, up), mu_s = dot(F.sun, up);
        const f3 tv = ray - up * mu_v, ts = F.sun - up * mu_s;
        const float nv = norm(tv), ns = norm(ts);
        const float cphi = (nv > 1e-6f && ns > 1e-6f) ? dot(tv, ts) / (nv * ns) : 1.0f;
        geometry_features(P, A.bottom, hs, mu_v, mu_s, cphi, fx);
        fx[4] = nets.lhr_n;
        fx[5] = nets.lhm_n;
        fx[6] = 2.0f * __logf(clampf(end - start, 1.0f, kSurrogateMaxLength)) / logf(kSurrogateMaxLength) - 1.0f;
        // twilight gate: the sun cosine small at the start, middle or end, or
        // of different signs there (the segment crosses the terminator)
        float mu_end, mu_mid;
        const float mu_min =
            mn(fabsf(mu_s), segment_features(P, A.bottom, G, ray, o_y, F.sun, start, end, fx, mu_end, mu_mid));
        const bool crosses = nets.gate_crossing && ((mu_s > 0.0f) != (mu_end > 0.0f) || (mu_s > 0.0f) != (mu_mid > 0.0f));
        kind = (mu_min < nets.twilight_cos || crosses) ? kSurfPlain : kSurfMlp;
      }
    } else if (nets.sky != nullptr && A.cam_alt <= P.top && fabsf(F.sun.y) >= nets.sky_twilight_cos && !near_limb) {
      kind = kSkyMlp;
      const float vl = sqrtf(ray.x * ray.x + ray.z * ray.z), sl = sqrtf(F.sun.x * F.sun.x + F.sun.z * F.sun.z);
      const float cphi = (vl > 1e-6f && sl > 1e-6f) ? (ray.x * F.sun.x + ray.z * F.sun.z) / (vl * sl) : 1.0f;
      geometry_features(P, A.bottom, A.cam_alt, ray.y, F.sun.y, cphi, fx);
      fx[4] = nets.lhr_n;
      fx[5] = nets.lhm_n;
      sky_ray_features(P, A.bottom, A.cam_alt, ray, F.sun, fx);
    } else {
      kind = kSkyLut;
    }
  }

  // the networks on the tensor cores, each run by the whole block when any
  // of its pixels needs it (block-uniform: every barrier stays convergent).
  // Tensor memory is taken only now, so that a block waiting for columns
  // has its features done, and not at all by a block without MLP pixels.
  // tc_ok is uniform over a tile; a tile whose wait timed out issues nothing
  // more and its MLP pixels take the plain path below.
  float yv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  bool tc_ok = true;
  const bool need_ap = __syncthreads_or(kind == kSurfMlp);
  const bool need_sky = __syncthreads_or(kind == kSkyMlp);
  // the weights have arrived (each thread observes the mbarrier before any
  // MMA of its tile reads them)
  const bool weights_ok = __syncthreads_and(tc::mbar_wait(&s_mbar[2], 0u, kTcWaitTries));
  if ((need_ap || need_sky) && weights_ok) {
    if (threadIdx.x < 32) tc::alloc(&s_tmem, kSurrogateTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    TcTile T{s_tmem + 128u * tile, s_tmem + 128u * tile + 64u, &s_mbar[tile], 0u, tile, int(threadIdx.x & 127)};
    if (need_ap) {
      float t[8];
      tc_ok = mlp_tile_tc<kSurrogateApHidden>(smem, kSurrogateApIn, T, fx, t, nets.wait_tries);
      if (kind == kSurfMlp)
        for (int k = 0; k < 8; ++k) yv[k] = t[k];
    }
    if (need_sky && tc_ok) {
      float t[8];
      tc_ok = mlp_tile_tc<kSurrogateSkyHidden>(smem + nets.ap_bytes, kSurrogateSkyIn, T, fx, t, nets.wait_tries);
      if (kind == kSkyMlp)
        for (int k = 0; k < 8; ++k) yv[k] = t[k];
    }
    // tensor memory is freed once no MMA is in flight: a tile that timed out
    // has exactly one commit outstanding, waited for here with the library's
    // full bound whatever the frame's own bound was
    tc::fence_before_sync();
    if (!tc_ok) tc::mbar_wait(T.mbar, T.phase ^ 1u, kTcWaitTries);
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x < 32) tc::dealloc(s_tmem, kSurrogateTmemCols);
  } else if (need_ap || need_sky) {
    tc_ok = false;  // the weights did not arrive in time
  }
  if (!tc_ok) {
    // the networks' outputs are not valid: the plain path for these pixels
    if (kind == kSurfMlp) kind = kSurfPlain;
    if (kind == kSkyMlp) kind = kSkyLut;
    if ((threadIdx.x & 127) == 0) atomicOr(Q.status, 1u);
  }

  bool queued = false;
  uint32_t qkind = kQueueSurface;
  f3 Lnet = mk(-1.0f, 0.0f, 0.0f);  // the network's in-scattering (x < 0: none)
  if (inside && kind != kSurfPlain) {
    f3 color = kShade ? shaded_scene(P, F, A, S, L, I, x, y, e, sid[e]) : ld3(scene + o);
    if (kind == kSurfMlp) {
      // transmittance: the plain path's own two-tap LUT ratio (:1603-1665);
      // in-scattering: the network, ln(L / E + floor + floor_t T)
      const f3 Tm = surface_segment_t(P, F, camera_ray_geom(P, A.bottom, A.cam_alt, ray), ray, start, end);
      const f3 Lm = net_radiance(yv, A.E, splat(nets.floor) + Tm * nets.floor_t);
      color = Lm + color * Tm;
      Lnet = Lm;
      if (check_pixel(x, y, Q.seed, Q.check_fraction)) {
        queued = true;
        qkind = kQueueSurfaceCheck;
      }
    } else if (kind == kSkyMlp) {
      const f3 sky = net_radiance(yv, A.E, splat(nets.sky_floor));
      color = composite_sky_with(P, F, A, sky, ray, color, ld3(space + o), float(L.height));
      if (check_pixel(x, y, Q.seed, Q.check_fraction)) {
        queued = true;
        qkind = kQueueSkyCheck;
      }
    } else if (kind == kSkyLut) {
      color = composite_sky(P, F, A, svlut, ray, color, ld3(space + o), float(L.height));
    }
    color = vmax(color, 0.0f);
    hdr[o + 0] = color.x;
    hdr[o + 1] = color.y;
    hdr[o + 2] = color.z;
  } else if (kind == kSurfPlain) {
    queued = true;
  }
  if (inside && Q.lm != nullptr) {  // the calibration's scratch: every pixel, each frame
    float* lm = Q.lm + 3 * storage_index(L, x, y);
    lm[0] = Lnet.x;
    if (Lnet.x >= 0.0f) {
      lm[1] = Lnet.y;
      lm[2] = Lnet.z;
    }
  }

  // warp-aggregated append to the fallback queue
  const int lane = threadIdx.x & 31;
  const unsigned qm = __ballot_sync(kAll, queued);
  if (qm) {
    const int leader = __ffs(qm) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(Q.count, uint32_t(__popc(qm)));
    base = __shfl_sync(kAll, base, leader);
    if (queued)
      Q.items[base + __popc(qm & ((1u << lane) - 1u))] = (qkind << 30) | uint32_t(cy * L.width + cx);
  }
  if (Q.stats != nullptr) {
    if (!tc_ok && (threadIdx.x & 127) == 0) atomicAdd(Q.stats + 7, 1.0f);  // tiles whose MMA timed out
    const unsigned gs = __ballot_sync(kAll, kind == kSurfPlain), ms = __ballot_sync(kAll, kind == kSurfMlp);
    const unsigned mk_ = __ballot_sync(kAll, kind == kSkyMlp), ls = __ballot_sync(kAll, kind == kSkyLut);
    if (lane == 0) {
      if (gs) atomicAdd(Q.stats + 3, float(__popc(gs)));
      if (ms) atomicAdd(Q.stats + 4, float(__popc(ms)));
      if (mk_) atomicAdd(Q.stats + 5, float(__popc(mk_)));
      if (ls) atomicAdd(Q.stats + 6, float(__popc(ls)));
    }
  }
}

// The plain integrator over the queued pixels: gated surface pixels get it
// as their result; checked pixels compare the MLP's color (in hdr) with it,
// then keep the plain result.  Warps take 32 entries per ticket.
template <bool kShade>
__global__ void __launch_bounds__(256, 2) k_surrogate_fallback(
    DevParams P, ImageLayout L, CompositeScalars A, const float* __restrict__ scene, const float* __restrict__ space,
    const float* __restrict__ pos, const float4* __restrict__ tlut, const float4* __restrict__ mslut,
    SurrogateQueue Q, float* __restrict__ hdr, unsigned long long* counter, ShadeParams S, ShadeImages I) {
  const Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
  const int lane = threadIdx.x & 31;
  const uint32_t n = *Q.count;
  uint32_t samples = 0, checked = 0;
  float err_sum = 0.0f, err_max = 0.0f;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(Q.count + 1, 32u);
    base = __shfl_sync(kAll, base, 0);
    if (base >= n) break;
    const uint32_t i = base + uint32_t(lane);
    if (i < n) {
      const uint32_t entry = Q.items[i];
      const uint32_t kind = entry >> 30, p = entry & 0x3fffffffu;
      const int x = int(p % uint32_t(L.width)), y = int(p / uint32_t(L.width));
      const size_t e = pix_offset(L, x, y);
      const size_t o = e * L.channels;
      const f3 ray = pixel_ray(L, A, x, y).ray;
      f3 color = kShade ? shaded_scene(P, F, A, S, L, I, x, y, e, I.surface_id[e]) : ld3(scene + o);
      if (kind == kQueueSkyCheck) {
        const f3 sky = sky_radiance(P, F, A.cam_alt, ray);
        samples += uint32_t(P.sv_steps);
        color = composite_sky_with(P, F, A, sky, ray, color, ld3(space + o), float(L.height));
      } else {
        float start, end;
        const RayGeom G = camera_ray_geom(P, A.bottom, A.cam_alt, ray);
        if (surface_interval(P, G, A.bottom, norm(ld3(pos + o)), start, end)) {
          const f3 Ls = integrate_surface(P, F, G, ray, start, end, samples);
          color = Ls + color * surface_segment_t(P, F, G, ray, start, end);
          if (kind == kQueueSurfaceCheck && Q.lm != nullptr) {
            // the calibration: this tile's log ratio of the plain in-scattering
            // to the network's; the pixel itself keeps the plain result
            float* lm = Q.lm + 3 * storage_index(L, x, y);
            const f3 Ln = ld3(lm);
            if (Ln.x >= 0.0f) {
              float* t = Q.tiles + 4 * ((y >> Q.tile_shift) * Q.tiles_x + (x >> Q.tile_shift));
              atomicAdd(t + 0, clampf(__logf(mx(Ls.x, 1e-12f) / mx(Ln.x, 1e-12f)), -kCalibrationClamp,
                                      kCalibrationClamp));
              atomicAdd(t + 1, clampf(__logf(mx(Ls.y, 1e-12f) / mx(Ln.y, 1e-12f)), -kCalibrationClamp,
                                      kCalibrationClamp));
              atomicAdd(t + 2, clampf(__logf(mx(Ls.z, 1e-12f) / mx(Ln.z, 1e-12f)), -kCalibrationClamp,
                                      kCalibrationClamp));
              atomicAdd(t + 3, 1.0f);
            }
            lm[0] = -1.0f;
          }
        }
      }
      color = vmax(color, 0.0f);
      if (kind != kQueueSurface) {
        const float err = color_error(ld3(hdr + o), color, F.E);
        ++checked;
        err_sum += err;
        err_max = mx(err_max, err);
      }
      hdr[o + 0] = color.x;
      hdr[o + 1] = color.y;
      hdr[o + 2] = color.z;
    }
  }
  warp_count(samples, counter);
  if (Q.stats != nullptr) {
    float c = float(checked);
#pragma unroll
    for (int k = 16; k > 0; k >>= 1) {
      c += __shfl_xor_sync(kAll, c, k);
      err_sum += __shfl_xor_sync(kAll, err_sum, k);
      err_max = mx(err_max, __shfl_xor_sync(kAll, err_max, k));
    }
    if (lane == 0 && c > 0.0f) {
      atomicAdd(Q.stats + 0, c);
      atomicAdd(Q.stats + 1, err_sum);
      atomicMax(reinterpret_cast<int*>(Q.stats + 2), __float_as_int(err_max));  // non-negative floats
    }
  }
}

// The calibration pass: every MLP surface pixel whose tile holds enough
// checked pixels gets its network in-scattering rescaled by the tile's mean
// log ratio, hdr += Lnet (exp(mean) - 1).  Thread per pixel in storage order.
__global__ void __launch_bounds__(256) k_surrogate_calibrate(ImageLayout L, SurrogateQueue Q, float* __restrict__ hdr) {
  const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i >= size_t(L.width) * size_t(L.height)) return;
  const float* lm = Q.lm + 3 * i;
  const float lx = lm[0];
  if (lx < 0.0f) return;
  int x, y;
  if (L.sy <= L.sx) {
    x = int(i / size_t(L.height));
    y = int(i % size_t(L.height));
  } else {
    y = int(i / size_t(L.width));
    x = int(i % size_t(L.width));
  }
  const float4 t = *reinterpret_cast<const float4*>(Q.tiles + 4 * ((y >> Q.tile_shift) * Q.tiles_x + (x >> Q.tile_shift)));
  if (t.w < float(kCalibrationMinChecks)) return;
  const float inv = 1.0f / t.w;
  const size_t o = pix_offset(L, x, y) * L.channels;
  hdr[o + 0] += lx * (__expf(t.x * inv) - 1.0f);
  hdr[o + 1] += lm[1] * (__expf(t.y * inv) - 1.0f);
  hdr[o + 2] += lm[2] * (__expf(t.z * inv) - 1.0f);
}

// Sky radiance of every pixel of a frame, the pixel's own view ray from the
// camera (the learned sky-view workload; the G-buffer is not read):
//  * kSkyPixelsPlain: the plain integrator per pixel - the sky-view march of
//    :1208-1302 (sv_steps warped segments) along the pixel's ray;
//  * kSkyPixelsNet: the sky network on the tensor cores; where a gate trips
//    (|sun cosine| at the camera below sky_twilight_cos, the view ray within
//    limb_rad of the limb, the camera above the shell) the plain integrator;
//  * kSkyPixelsLut: the reference's own path, a bilinear tap of the sky-view
//    LUT (:1474-1525).
// 256 threads = two 128-pixel tiles, as in k_composite_surrogate.
enum : int { kSkyPixelsPlain = 0, kSkyPixelsNet = 1, kSkyPixelsLut = 2 };
template <int kMode>
__global__ void __launch_bounds__(256, 2) k_sky_pixels(DevParams P, ImageLayout L, CompositeScalars A,
                                                       const float4* __restrict__ tlut,
                                                       const float4* __restrict__ mslut,
                                                       const float4* __restrict__ svlut, SurrogateNets nets,
                                                       uint32_t* __restrict__ status, float* __restrict__ out,
                                                       unsigned long long* counter, SurrogateQueue Q) {
  extern __shared__ __align__(128) unsigned char smem[];  // the sky network (kSkyPixelsNet)
  __shared__ __align__(8) uint64_t s_mbar[3];
  __shared__ uint32_t s_tmem;
  if (kMode == kSkyPixelsNet) {
    if (threadIdx.x == 0) {
      tc::mbar_init(&s_mbar[0], 1);
      tc::mbar_init(&s_mbar[1], 1);
      tc::mbar_init(&s_mbar[2], 1);
      tc::mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::mbar_arrive_expect_tx(&s_mbar[2], uint32_t(nets.sky_bytes));
      tc::bulk_g2s(smem, nets.sky, uint32_t(nets.sky_bytes), &s_mbar[2]);
    }
  }
  int x, y;
  const bool inside = tile_pixel(L, x, y);
  const int cx = inside ? x : 0, cy = inside ? y : 0;
  const Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
  const f3 ray = pixel_ray(L, A, cx, cy).ray;
  uint32_t samples = 0;
  f3 sky = splat(0.0f);
  bool plain = kMode == kSkyPixelsPlain;
  bool checked = false;
  if (kMode == kSkyPixelsLut) sky = sample_sky_view(P, svlut, ray, F.sun, A.sky_alt, A.bottom);
  if (kMode == kSkyPixelsNet) {
    const bool near_limb =
        fabsf(acosf(clampf(ray.y, -1.0f, 1.0f)) - sky_horizon_zenith(A.cam_alt, A.bottom)) < nets.limb_rad;
    const bool net = inside && A.cam_alt <= P.top && fabsf(F.sun.y) >= nets.sky_twilight_cos && !near_limb;
    plain = !net;
    float fx[16] = {};
    if (net) {
      const float vl = sqrtf(ray.x * ray.x + ray.z * ray.z), sl = sqrtf(F.sun.x * F.sun.x + F.sun.z * F.sun.z);
      const float cphi = (vl > 1e-6f && sl > 1e-6f) ? (ray.x * F.sun.x + ray.z * F.sun.z) / (vl * sl) : 1.0f;
      geometry_features(P, A.bottom, A.cam_alt, ray.y, F.sun.y, cphi, fx);
      fx[4] = nets.lhr_n;
      fx[5] = nets.lhm_n;
      sky_ray_features(P, A.bottom, A.cam_alt, ray, F.sun, fx);
    }
    const bool need = __syncthreads_or(net);
    const bool weights_ok = __syncthreads_and(tc::mbar_wait(&s_mbar[2], 0u, kTcWaitTries));
    bool tc_ok = weights_ok;
    float yv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (need && weights_ok) {
      if (threadIdx.x < 32) tc::alloc(&s_tmem, kSurrogateTmemCols);
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      const int tile = threadIdx.x >> 7;
      TcTile T{s_tmem + 128u * tile, s_tmem + 128u * tile + 64u, &s_mbar[tile], 0u, tile, int(threadIdx.x & 127)};
      tc_ok = mlp_tile_tc<kSurrogateSkyHidden>(smem, kSurrogateSkyIn, T, fx, yv, nets.wait_tries);
      tc::fence_before_sync();
      if (!tc_ok) tc::mbar_wait(T.mbar, T.phase ^ 1u, kTcWaitTries);
      __syncthreads();
      tc::fence_after_sync();
      if (threadIdx.x < 32) tc::dealloc(s_tmem, kSurrogateTmemCols);
    }
    if (need && !tc_ok) {
      plain = true;  // the network's outputs are not valid: the plain integrator
      if ((threadIdx.x & 127) == 0) atomicOr(status, 1u);
    } else if (net) {
      sky = net_radiance(yv, A.E, splat(nets.sky_floor));
      checked = Q.net_mask != nullptr && check_pixel(x, y, Q.seed, Q.check_fraction);
    }
  }
  if (inside) {
    if (plain) {
      sky = sky_radiance(P, F, A.cam_alt, ray);
      samples = uint32_t(P.sv_steps);
    }
    const size_t o = pix_offset(L, x, y) * L.channels;
    out[o + 0] = sky.x;
    out[o + 1] = sky.y;
    out[o + 2] = sky.z;
    if (kMode == kSkyPixelsNet && Q.net_mask != nullptr)  // the calibration: which pixels are the network's
      Q.net_mask[storage_index(L, x, y)] = plain ? 0 : 1;
  }
  if (kMode == kSkyPixelsNet) {  // checked network pixels to the queue (warp-aggregated)
    const int lane = threadIdx.x & 31;
    const unsigned qm = __ballot_sync(kAll, checked);
    if (qm) {
      const int leader = __ffs(qm) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(Q.count, uint32_t(__popc(qm)));
      base = __shfl_sync(kAll, base, leader);
      if (checked)
        Q.items[base + __popc(qm & ((1u << lane) - 1u))] = (kQueueSkyCheck << 30) | uint32_t(cy * L.width + cx);
    }
  }
  warp_count(samples, counter);
}

// The sky-pixel calibration pass: every network pixel of a tile holding
// enough checked pixels is scaled by the tile's mean ratio.  Thread per
// pixel in storage order.
__global__ void __launch_bounds__(256) k_sky_pixels_calibrate(ImageLayout L, SurrogateQueue Q, float* __restrict__ out) {
  const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i >= size_t(L.width) * size_t(L.height) || Q.net_mask[i] == 0) return;
  int x, y;
  if (L.sy <= L.sx) {
    x = int(i / size_t(L.height));
    y = int(i % size_t(L.height));
  } else {
    y = int(i / size_t(L.width));
    x = int(i % size_t(L.width));
  }
  const float4 t = *reinterpret_cast<const float4*>(Q.tiles + 4 * ((y >> Q.tile_shift) * Q.tiles_x + (x >> Q.tile_shift)));
  if (t.w < float(kCalibrationMinChecks)) return;
  const float inv = 1.0f / t.w;
  const size_t o = pix_offset(L, x, y) * L.channels;
  out[o + 0] *= __expf(t.x * inv);
  out[o + 1] *= __expf(t.y * inv);
  out[o + 2] *= __expf(t.z * inv);
}

// The sky-pixel calibration's checks: each queued network pixel gets the
// plain march, adds its tile's log ratio of plain to network radiance, and
// keeps the plain result.  Warps take 32 entries per ticket.
__global__ void __launch_bounds__(256) k_sky_pixels_check(DevParams P, ImageLayout L, CompositeScalars A,
                                                          const float4* __restrict__ tlut,
                                                          const float4* __restrict__ mslut, SurrogateQueue Q,
                                                          float* __restrict__ out, unsigned long long* counter) {
  const Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
  const int lane = threadIdx.x & 31;
  const uint32_t n = *Q.count;
  uint32_t samples = 0;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(Q.count + 1, 32u);
    base = __shfl_sync(kAll, base, 0);
    if (base >= n) break;
    const uint32_t i = base + uint32_t(lane);
    if (i < n) {
      const uint32_t p = Q.items[i] & 0x3fffffffu;
      const int x = int(p % uint32_t(L.width)), y = int(p / uint32_t(L.width));
      const f3 ray = pixel_ray(L, A, x, y).ray;
      const f3 sky = sky_radiance(P, F, A.cam_alt, ray);
      samples += uint32_t(P.sv_steps);
      const size_t o = pix_offset(L, x, y) * L.channels;
      const f3 Ln = ld3(out + o);  // the network's radiance
      float* t = Q.tiles + 4 * ((y >> Q.tile_shift) * Q.tiles_x + (x >> Q.tile_shift));
      atomicAdd(t + 0, clampf(__logf(mx(sky.x, 1e-12f) / mx(Ln.x, 1e-12f)), -kCalibrationClamp, kCalibrationClamp));
      atomicAdd(t + 1, clampf(__logf(mx(sky.y, 1e-12f) / mx(Ln.y, 1e-12f)), -kCalibrationClamp, kCalibrationClamp));
      atomicAdd(t + 2, clampf(__logf(mx(sky.z, 1e-12f) / mx(Ln.z, 1e-12f)), -kCalibrationClamp, kCalibrationClamp));
      atomicAdd(t + 3, 1.0f);
      Q.net_mask[storage_index(L, x, y)] = 0;
      out[o + 0] = sky.x;
      out[o + 1] = sky.y;
      out[o + 2] = sky.z;
    }
  }
  warp_count(samples, counter);
}

}  // namespace

cudaError_t launch_sky_pixels(int mode, const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                              const float4* tlut, const float4* mslut, const float4* svlut, const SurrogateNets& nets,
                              uint32_t* status, float* out, unsigned long long* counter, int sm_count, cudaStream_t s,
                              const SurrogateQueue* calibration) {
  const dim3 grid((L.width + 15) / 16, (L.height + 15) / 16);
  SurrogateQueue Q{};
  if (mode == kSkyPixelsNet && calibration != nullptr && calibration->net_mask != nullptr) Q = *calibration;
  if (mode == kSkyPixelsNet) {
    cudaError_t e = cudaFuncSetAttribute(k_sky_pixels<kSkyPixelsNet>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         nets.sky_bytes);
    if (e != cudaSuccess) return e;
    if (Q.net_mask != nullptr) {
      const int tiles_y = (L.height + (1 << Q.tile_shift) - 1) >> Q.tile_shift;
      e = cudaMemsetAsync(Q.count, 0, 2 * sizeof(uint32_t), s);
      if (e == cudaSuccess) e = cudaMemsetAsync(Q.tiles, 0, sizeof(float) * 4 * size_t(Q.tiles_x) * tiles_y, s);
      if (e != cudaSuccess) return e;
    }
    k_sky_pixels<kSkyPixelsNet><<<grid, 256, nets.sky_bytes, s>>>(P, L, A, tlut, mslut, svlut, nets, status, out,
                                                                  counter, Q);
    e = cudaGetLastError();
    if (e != cudaSuccess || Q.net_mask == nullptr) return e;
    k_sky_pixels_check<<<2 * sm_count, 256, 0, s>>>(P, L, A, tlut, mslut, Q, out, counter);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t pixels = size_t(L.width) * L.height;
    k_sky_pixels_calibrate<<<unsigned((pixels + 255) / 256), 256, 0, s>>>(L, Q, out);
  } else if (mode == kSkyPixelsLut) {
    k_sky_pixels<kSkyPixelsLut><<<grid, 256, 0, s>>>(P, L, A, tlut, mslut, svlut, nets, status, out, counter, Q);
  } else {
    k_sky_pixels<kSkyPixelsPlain><<<grid, 256, 0, s>>>(P, L, A, tlut, mslut, svlut, nets, status, out, counter, Q);
  }
  return cudaGetLastError();
}

cudaError_t launch_gen_samples(const SurrogateSetDev* sets, int n_sets, int kind, long long n, unsigned long long seed,
                               const SampleShaping& shaping, const float E[3], float ar, float* features,
                               float* targets, unsigned long long* counter, cudaStream_t s) {
  const f3 e3 = {E[0], E[1], E[2]};
  k_gen_samples<<<unsigned((n + 127) / 128), 128, 0, s>>>(sets, n_sets, kind, n, seed, shaping, e3, ar, features,
                                                         targets, counter);
  return cudaGetLastError();
}

size_t surrogate_smem_bytes(const SurrogateNets& nets) { return size_t(nets.ap_bytes) + size_t(nets.sky_bytes); }

cudaError_t launch_composite_surrogate(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                                       const float* scene, const float* space, const int32_t* sid, const float* pos,
                                       const float4* tlut, const float4* mslut, const float4* svlut,
                                       const SurrogateNets& nets, const SurrogateQueue& Q, float* hdr,
                                       unsigned long long* counter, int sm_count, cudaStream_t s,
                                       const ShadeParams* shade, const ShadeImages* shade_images) {
  cudaError_t e = cudaMemsetAsync(Q.count, 0, 2 * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const int tiles_y = (L.height + (1 << Q.tile_shift) - 1) >> Q.tile_shift;
  if (Q.lm != nullptr) {
    e = cudaMemsetAsync(Q.tiles, 0, sizeof(float) * 4 * size_t(Q.tiles_x) * tiles_y, s);
    if (e != cudaSuccess) return e;
  }
  const int smem = int(surrogate_smem_bytes(nets));
  const dim3 grid((L.width + 15) / 16, (L.height + 15) / 16);
  const ShadeParams S = shade ? *shade : ShadeParams{};
  const ShadeImages I = shade_images ? *shade_images : ShadeImages{};
  if (shade) {
    e = cudaFuncSetAttribute(k_composite_surrogate<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_composite_surrogate<true><<<grid, 256, smem, s>>>(P, L, A, scene, space, sid, pos, tlut, mslut, svlut, nets, Q,
                                                        hdr, S, I);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_surrogate_fallback<true><<<2 * sm_count, 256, 0, s>>>(P, L, A, scene, space, pos, tlut, mslut, Q, hdr, counter,
                                                            S, I);
  } else {
    e = cudaFuncSetAttribute(k_composite_surrogate<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_composite_surrogate<false><<<grid, 256, smem, s>>>(P, L, A, scene, space, sid, pos, tlut, mslut, svlut, nets,
                                                         Q, hdr, S, I);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_surrogate_fallback<false><<<2 * sm_count, 256, 0, s>>>(P, L, A, scene, space, pos, tlut, mslut, Q, hdr,
                                                             counter, S, I);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess || Q.lm == nullptr) return e;
  const size_t pixels = size_t(L.width) * L.height;
  k_surrogate_calibrate<<<unsigned((pixels + 255) / 256), 256, 0, s>>>(L, Q, hdr);
  return cudaGetLastError();
}

}  // namespace atm
