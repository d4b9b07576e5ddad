// atm_ocean.cu - the ocean coverage pass that completes the G-buffer before
// the atmosphere stage (OceanRenderer, src/planet_renderer/ocean.py:193-771)
// on sm_103a:
//
//  * k_ocean_spectrum: thread per texel of the three periodic cascades: the
//    12-mode directional wave sum of _build_directional_spectrum (:260-337)
//    into height + gradient, horizontal displacement and its Jacobian;
//  * k_ocean_coverage: thread per pixel along the image's contiguous axis:
//    the view ray against the sea-level sphere (_near_sphere_distance), the
//    reseed from the outer sphere, three fixed-point solves against the
//    displaced surface within geometry_max_distance, then, where the sea is
//    nearer than the terrain, the water surface's G-buffer: view position,
//    footprint-filtered wave normal, unresolved slope variance, seabed
//    colour / normal / water depth from the terrain pixel it covers
//    (_rasterize :517-684).
//
// Arithmetic is IEEE float32 in the reference's operation order without
// contraction (atm_f32.cuh).  The spectrum's sines and cosines are CUDA's
// sinf / cosf, whose last bit may differ from the reference runtime's, so
// values agree to float32 rounding rather than bit for bit.
#include <cuda_runtime.h>

#include <cstdint>

#include "atm_f32.cuh"
#include "atm_kernels.h"

namespace atm {

namespace {

using namespace f32;

// The spectrum's table (ocean.py:18-25), each value rounded from its double
// literal to float32 as the reference's Taichi vectors round it.
constexpr int kModes = 12;
constexpr double kWeightSum = 1.0 + 0.82 + 0.72 + 0.60 + 0.52 + 0.68 + 0.55 + 0.42 + 0.36 + 0.31 + 0.27 + 0.22;
constexpr double kPi = 3.141592653589793;
__constant__ float kPeriods[kOceanCascades] = {2048.0f, 256.0f, 32.0f};
__constant__ float kHeights[kOceanCascades] = {float(0.62), float(0.14), float(0.025)};
__constant__ float kModeX[kModes] = {3, 4, 4, 5, 5, 3, 2, 1, -1, -2, -3, -4};
__constant__ float kModeY[kModes] = {1, 1, 2, 1, 2, 2, 3, 4, 4, 3, 2, 1};
__constant__ float kWeights[kModes] = {1.0f,        float(0.82), float(0.72), float(0.60), float(0.52), float(0.68),
                                       float(0.55), float(0.42), float(0.36), float(0.31), float(0.27), float(0.22)};
__constant__ float kPhases[kModes] = {float(0.31), float(1.73), float(3.11), float(4.67), float(0.93), float(2.39),
                                      float(5.21), float(3.83), float(1.17), float(5.72), float(2.83), float(4.09)};

// _build_directional_spectrum :260-337
__global__ void __launch_bounds__(256) k_ocean_spectrum(OceanSpectrum S, float time_s, float amplitude_scale,
                                                        float choppiness) {
  const int n = S.n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kOceanCascades * n * n) return;
  const int c = i / (n * n), x = (i / n) % n, y = i % n;
  const float two_pi = float(2.0 * kPi), pi = float(kPi);
  const float period = kPeriods[c];
  const float u = dv(add(float(x), 0.5f), float(n)), v = dv(add(float(y), 0.5f), float(n));
  float h = 0.0f, gx = 0.0f, gy = 0.0f, dx = 0.0f, dy = 0.0f, j0 = 0.0f, j1 = 0.0f, j2 = 0.0f, j3 = 0.0f;
#pragma unroll
  for (int m = 0; m < kModes; ++m) {
    const float kx = kModeX[m], ky = kModeY[m];
    const float mode_length = __fsqrt_rn(add(mul(kx, kx), mul(ky, ky)));
    const float wave_number = dv(mul(two_pi, mode_length), period);
    const float omega = __fsqrt_rn(mul(float(9.81), wave_number));
    const float phase = sub(add(mul(two_pi, add(mul(kx, u), mul(ky, v))), kPhases[m]), mul(omega, time_s));
    const float amplitude = dv(mul(mul(kHeights[c], amplitude_scale), kWeights[m]),
                               float(kWeightSum));
    const float cp = cosf(phase), sp = sinf(phase);
    h = add(h, mul(amplitude, cp));
    const float derivative = mul(mul(mul(-amplitude, sp), 2.0f), pi);
    gx = add(gx, dv(mul(derivative, kx), period));
    gy = add(gy, dv(mul(derivative, ky), period));
    const float len = fmx(mode_length, float(1.0e-6));
    const float dirx = dv(kx, len), diry = dv(ky, len);
    const float wvx = dv(mul(two_pi, kx), period), wvy = dv(mul(two_pi, ky), period);
    const float choppy = mul(choppiness, amplitude);
    const float ds = mul(-choppy, sp);
    dx = add(dx, mul(ds, dirx));
    dy = add(dy, mul(ds, diry));
    const float js = mul(-choppy, cp);
    j0 = add(j0, mul(js, mul(dirx, wvx)));
    j1 = add(j1, mul(js, mul(dirx, wvy)));
    j2 = add(j2, mul(js, mul(diry, wvx)));
    j3 = add(j3, mul(js, mul(diry, wvy)));
  }
  S.height_gradient[i] = make_float4(h, gx, gy, 0.0f);
  S.displacement[i] = make_float2(dx, dy);
  S.jacobian[i] = make_float4(j0, j1, j2, j3);
}

__device__ __forceinline__ float lerp_ref(float a, float b, float f) { return add(mul(a, sub(1.0f, f)), mul(b, f)); }

// _sample_spectrum_texture :383-425: periodic bilinear taps of one cascade.
struct Taps {
  int i00, i10, i01, i11;
  float fx, fy;
};
__device__ __forceinline__ Taps spectrum_taps(int n, int cascade, float u, float v) {
  const float wu = sub(u, floorf(u)), wv = sub(v, floorf(v));
  const float tu = sub(mul(wu, float(n)), 0.5f), tv = sub(mul(wv, float(n)), 0.5f);
  const float bu = floorf(tu), bv = floorf(tv);
  const int bx = int(bu), by = int(bv);  // NaN converts to 0; the wrap keeps every index in range
  Taps t;
  t.fx = sub(tu, float(bx));
  t.fy = sub(tv, float(by));
  const int x0 = ((bx % n) + n) % n, y0 = ((by % n) + n) % n;
  const int x1 = (x0 + 1) % n, y1 = (y0 + 1) % n;
  const int base = cascade * n * n;
  t.i00 = base + x0 * n + y0;
  t.i10 = base + x1 * n + y0;
  t.i01 = base + x0 * n + y1;
  t.i11 = base + x1 * n + y1;
  return t;
}
__device__ __forceinline__ float2 taps_disp(const OceanSpectrum& S, const Taps& t) {
  const float2 a = __ldg(S.displacement + t.i00), b = __ldg(S.displacement + t.i10), c = __ldg(S.displacement + t.i01),
               d = __ldg(S.displacement + t.i11);
  return make_float2(lerp_ref(lerp_ref(a.x, b.x, t.fx), lerp_ref(c.x, d.x, t.fx), t.fy),
                     lerp_ref(lerp_ref(a.y, b.y, t.fx), lerp_ref(c.y, d.y, t.fx), t.fy));
}
__device__ __forceinline__ float4 lerp4(const float4* p, const Taps& t) {
  const float4 a = __ldg(p + t.i00), b = __ldg(p + t.i10), c = __ldg(p + t.i01), d = __ldg(p + t.i11);
  return make_float4(lerp_ref(lerp_ref(a.x, b.x, t.fx), lerp_ref(c.x, d.x, t.fx), t.fy),
                     lerp_ref(lerp_ref(a.y, b.y, t.fx), lerp_ref(c.y, d.y, t.fx), t.fy),
                     lerp_ref(lerp_ref(a.z, b.z, t.fx), lerp_ref(c.z, d.z, t.fx), t.fy),
                     lerp_ref(lerp_ref(a.w, b.w, t.fx), lerp_ref(c.w, d.w, t.fx), t.fy));
}

// _cascade_axes :364-381 (global sampling axes rotated by the wind)
__device__ __forceinline__ void cascade_axes(int c, float cw, float sw, r3& au, r3& av) {
  const r3 bu = c == 0 ? R3(1.0f, 0.0f, 0.0f) : (c == 1 ? R3(0.0f, 1.0f, 0.0f) : R3(0.0f, 0.0f, 1.0f));
  const r3 bv = c == 0 ? R3(0.0f, 0.0f, 1.0f) : (c == 1 ? R3(1.0f, 0.0f, 0.0f) : R3(0.0f, 1.0f, 0.0f));
  au = radd(rscale(bu, cw), rscale(bv, sw));
  av = radd(rscale(R3(-bu.x, -bu.y, -bu.z), sw), rscale(bv, cw));
}

// The undisturbed coordinate of cascade c under the displaced point: the
// Gerstner map inverted by two fixed-point steps (:448-468).
__device__ __forceinline__ Taps inverted_taps(const OceanSpectrum& S, const OceanFrame& F, int c, r3 goff, r3 au,
                                              r3 av) {
  const float period = kPeriods[c];
  const float bu = add(F.offsets[c][0], dv(rdot(goff, au), period));
  const float bv = add(F.offsets[c][1], dv(rdot(goff, av), period));
  float u = bu, v = bv;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const float2 d = taps_disp(S, spectrum_taps(S.n, c, u, v));
    u = sub(bu, dv(d.x, period));
    v = sub(bv, dv(d.y, period));
  }
  return spectrum_taps(S.n, c, u, v);
}

// _sample_spectrum(geometry_only=True): summed height of the geometry cascades
__device__ float wave_height(const OceanSpectrum& S, const OceanFrame& F, r3 goff, float cw, float sw) {
  float height = 0.0f;
  for (int c = 0; c < kOceanCascades; ++c) {
    if (c >= F.geometry_cascades) break;
    r3 au, av;
    cascade_axes(c, cw, sw, au, av);
    const Taps t = inverted_taps(S, F, c, goff, au, av);
    height = add(height, lerp4(S.height_gradient, t).x);
  }
  return height;
}

// _sample_spectrum(geometry_only=False): the footprint-resolved slope and the
// unresolved slope variance of all cascades
__device__ void wave_slope(const OceanSpectrum& S, const OceanFrame& F, r3 goff, r3 radial, float footprint, float cw,
                           float sw, r3& slope, float& unresolved) {
  slope = R3(0.0f, 0.0f, 0.0f);
  unresolved = 0.0f;
  for (int c = 0; c < kOceanCascades; ++c) {
    r3 au, av;
    cascade_axes(c, cw, sw, au, av);
    const Taps t = inverted_taps(S, F, c, goff, au, av);
    const float4 hg = lerp4(S.height_gradient, t);
    const float4 j = lerp4(S.jacobian, t);
    const float min_wavelength = dv(kPeriods[c], 5.5f);
    const float spw = dv(min_wavelength, fmx(footprint, 0.01f));
    float resolved = fmn(fmx(dv(sub(spw, 2.0f), 4.0f), 0.0f), 1.0f);
    resolved = mul(mul(resolved, resolved), sub(3.0f, mul(2.0f, resolved)));
    const float m00 = add(1.0f, j.x), m01 = j.y, m10 = j.z, m11 = add(1.0f, j.w);
    const float det = sub(mul(m00, m11), mul(m01, m10));
    const float safe = fabsf(det) < 0.15f ? (det >= 0.0f ? 0.15f : -0.15f) : det;
    const float mg0 = dv(sub(mul(m11, hg.y), mul(m10, hg.z)), safe);
    const float mg1 = dv(add(mul(-m01, hg.y), mul(m00, hg.z)), safe);
    const r3 tu = rsub(au, rscale(radial, rdot(radial, au)));
    const r3 tv = rsub(av, rscale(radial, rdot(radial, av)));
    slope = radd(slope, rscale(radd(rscale(tu, mg0), rscale(tv, mg1)), resolved));
    unresolved = add(unresolved, mul(F.variances[c], sub(1.0f, mul(resolved, resolved))));
  }
}

// _near_sphere_distance :339-362
__device__ __forceinline__ float near_sphere_distance(float altitude, float ray_cosine, float radius) {
  const float origin_radius = add(radius, altitude);
  const float half_linear = mul(origin_radius, ray_cosine);
  const float constant = mul(altitude, add(mul(2.0f, radius), altitude));
  const float disc = sub(mul(half_linear, half_linear), constant);
  float distance = -1.0f;
  if (disc >= 0.0f) {
    const float root = __fsqrt_rn(fmx(disc, 0.0f));
    const float q = sub(-half_linear, half_linear >= 0.0f ? root : -root);
    float root0 = sub(-half_linear, root), root1 = add(-half_linear, root);
    if (fabsf(q) > float(1.0e-12)) {
      root0 = q;
      root1 = dv(constant, q);
    }
    const float nearer = fmn(root0, root1), farther = fmx(root0, root1);
    if (nearer > 0.0f)
      distance = nearer;
    else if (farther > 0.0f)
      distance = farther;
  }
  return distance;
}

__device__ __forceinline__ float rnorm(r3 v) { return __fsqrt_rn(rdot(v, v)); }
__device__ __forceinline__ r3 rdiv(r3 v, float s) { return {dv(v.x, s), dv(v.y, s), dv(v.z, s)}; }
__device__ __forceinline__ r3 ld3(const float* p) { return R3(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(float* p, r3 v) {
  p[0] = v.x;
  p[1] = v.y;
  p[2] = v.z;
}

// _rasterize :517-684
__global__ void __launch_bounds__(256) k_ocean_coverage(OceanSpectrum S, OceanFrame F, ImageLayout L,
                                                        OceanImages G) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)L.width * L.height) return;
  int x, y;
  if (L.sy <= L.sx) {
    x = int(i / L.height);
    y = int(i % L.height);
  } else {
    y = int(i / L.width);
    x = int(i % L.width);
  }
  const r3 east = R3(F.east[0], F.east[1], F.east[2]), up = R3(F.up[0], F.up[1], F.up[2]),
           north = R3(F.north[0], F.north[1], F.north[2]);
  const float aspect = dv(float(L.width), float(L.height));
  const float su = dv(add(float(x), 0.5f), float(L.width)), sv = dv(add(float(y), 0.5f), float(L.height));
  const float sx = mul(sub(mul(su, 2.0f), 1.0f), aspect), sy = sub(mul(sv, 2.0f), 1.0f);
  const r3 ray_view = rnormalized(R3(sx, sy, dv(1.0f, F.tf)));
  const r3 ray_local = radd(radd(rscale(R3(F.right[0], F.right[1], F.right[2]), ray_view.x),
                                 rscale(R3(F.vup[0], F.vup[1], F.vup[2]), ray_view.y)),
                            rscale(R3(F.fwd[0], F.fwd[1], F.fwd[2]), ray_view.z));
  const float R = F.radius, alt = F.altitude;
  float distance = near_sphere_distance(alt, ray_local.y, R);
  if (distance <= 0.1f && F.max_displacement > 0.0f && alt > F.max_displacement)
    distance = near_sphere_distance(sub(alt, F.max_displacement), ray_local.y, add(R, F.max_displacement));
  const r3 origin = R3(0.0f, add(R, alt), 0.0f);
  const float cw = cosf(F.wind), sw = sinf(F.wind);
  auto to_global = [&](r3 v) { return radd(radd(rscale(east, v.x), rscale(up, v.y)), rscale(north, v.z)); };
  auto offset_global = [&](r3 v) {
    return radd(radd(rscale(east, v.x), rscale(up, sub(v.y, R))), rscale(north, v.z));
  };
  if (distance > 0.1f && distance <= F.geometry_max_distance) {
    for (int it = 0; it < 3; ++it) {
      const r3 cand = radd(origin, rscale(ray_local, distance));
      const float h = wave_height(S, F, offset_global(cand), cw, sw);
      const float displaced = near_sphere_distance(sub(alt, h), ray_local.y, add(R, h));
      if (displaced > 0.1f) distance = displaced;
    }
  }
  if (!(distance > 0.1f)) return;
  const long long e = (long long)x * L.sx + (long long)y * L.sy;
  const int c = L.channels;
  const r3 ocean_view = rscale(ray_view, distance);
  const int32_t sid = G.surface_id[e];
  if (!(sid < 0 || ocean_view.z < G.depth[e])) return;
  const float max_depth = F.max_visible_depth;
  float seabed_distance = add(distance, max_depth);
  r3 seabed_color = R3(0.025f, 0.035f, 0.025f);
  r3 seabed_normal = R3(0.0f, 1.0f, 0.0f);
  const bool has_seabed = sid >= 0;
  if (has_seabed) {
    seabed_distance = rnorm(ld3(G.position + e * c));
    seabed_color = ld3(G.albedo + e * c);
    seabed_normal = ld3(G.normal + e * c);
  }
  const float optical_depth = fmn(fmx(sub(seabed_distance, distance), 0.0f), max_depth);
  const r3 ocean_local = radd(origin, rscale(ray_local, distance));
  const float ocean_norm = rnorm(ocean_local);
  const r3 radial_global = rnormalized(to_global(rdiv(ocean_local, fmx(ocean_norm, 1.0f))));
  if (!has_seabed) seabed_normal = radial_global;
  const float footprint = dv(mul(mul(distance, 2.0f), F.tf), float(L.height));
  r3 slope = R3(0.0f, 0.0f, 0.0f);
  float unresolved = 0.0f;
  if (F.enabled) wave_slope(S, F, offset_global(ocean_local), radial_global, footprint, cw, sw, slope, unresolved);
  const r3 water_normal = rnormalized(rsub(radial_global, rscale(slope, F.normal_strength)));
  r3 color = R3(F.albedo[0], F.albedo[1], F.albedo[2]);
  if (F.debug_mode == 1)
    color = R3(0.02f, 0.63f, 0.82f);
  else if (F.debug_mode == 2)
    color = R3(0.05f, 0.18f, 0.70f);
  else if (F.debug_mode == 3)
    color = R3(0.04f, 0.35f, 0.62f);
  G.depth[e] = ocean_view.z;
  st3(G.position + e * c, ocean_view);
  st3(G.normal + e * c, water_normal);
  st3(G.albedo + e * c, color);
  for (int k = 0; k < 4; ++k) G.material[e * 4 + k] = 0.0f;
  G.height[e] = sub(ocean_norm, R);
  G.water_depth[e] = optical_depth;
  st3(G.seabed_albedo + e * c, seabed_color);
  st3(G.seabed_normal + e * c, seabed_normal);
  G.slope_variance[e] = unresolved;
  G.surface_id[e] = kOceanSurfaceId;
  G.cell_id[e] = -1;
}

}  // namespace

cudaError_t launch_ocean_spectrum(const OceanSpectrum& S, float time_s, float amplitude_scale, float choppiness,
                                  cudaStream_t s) {
  const int texels = kOceanCascades * S.n * S.n;
  k_ocean_spectrum<<<(texels + 255) / 256, 256, 0, s>>>(S, time_s, amplitude_scale, choppiness);
  return cudaGetLastError();
}

cudaError_t launch_ocean_coverage(const OceanSpectrum& S, const OceanFrame& F, const ImageLayout& L,
                                  const OceanImages& G, cudaStream_t s) {
  const long long pixels = (long long)L.width * L.height;
  k_ocean_coverage<<<unsigned((pixels + 255) / 256), 256, 0, s>>>(S, F, L, G);
  return cudaGetLastError();
}

}  // namespace atm
