// atm_shade.cuh - the surface shading of one pixel (PlanetRenderer._shade_surface,
// src/planet_renderer/renderer.py :1277-1575) as a device function, shared
// by the shading kernel and the fused frame kernels: Lambertian land under
// the transmitted sun and the sky radiance; ocean pixels (advanced ocean on)
// with a GGX-style sun specular, Fresnel sky reflection and a water body
// over a seabed reconstructed along the refracted view ray from the opaque
// terrain snapshot (bilinear over four neighbours, depth-tested).
// Arithmetic is IEEE float32 in the reference's operation order without
// contraction (__fmul_rn / __fadd_rn), so results follow the reference's to
// the last bits of expf.
#pragma once

#include <cstdint>

#include "atm_kernels.h"

namespace atm {
namespace shading {

struct v3 {
  float x, y, z;
};
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fmx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fmn(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ v3 V(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ v3 vadd(v3 a, v3 b) { return {add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)}; }
__device__ __forceinline__ v3 vsub(v3 a, v3 b) { return {sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)}; }
__device__ __forceinline__ v3 vmul(v3 a, v3 b) { return {mul(a.x, b.x), mul(a.y, b.y), mul(a.z, b.z)}; }
__device__ __forceinline__ v3 vscale(v3 a, float s) { return {mul(a.x, s), mul(a.y, s), mul(a.z, s)}; }
__device__ __forceinline__ v3 vdivs(v3 a, float s) { return {dv(a.x, s), dv(a.y, s), dv(a.z, s)}; }
__device__ __forceinline__ v3 vneg(v3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ v3 vmax0(v3 a) { return {fmx(a.x, 0.0f), fmx(a.y, 0.0f), fmx(a.z, 0.0f)}; }
__device__ __forceinline__ float vdot(v3 a, v3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
__device__ __forceinline__ float vnorm(v3 a) { return __fsqrt_rn(vdot(a, a)); }
// Taichi's normalized(): (1 / |v|) * v
__device__ __forceinline__ v3 vunit(v3 a) {
  const float inv = dv(1.0f, vnorm(a));
  return {mul(inv, a.x), mul(inv, a.y), mul(inv, a.z)};
}
__device__ __forceinline__ v3 ld(const float* p, int64_t e, int c) { return {p[e * c], p[e * c + 1], p[e * c + 2]}; }
__device__ __forceinline__ v3 cv(const float (&a)[3]) { return {a[0], a[1], a[2]}; }

constexpr float kPi = 3.14159265358979323846f;  // f32(math.pi)

// The shaded colour of pixel (x, y) (element e, surface id sid) given its
// sun transmittance T and sky radiance at the surface (the surface lighting
// of prepare_frame); sky pixels (sid < 0) get the reference's background.
// Not clamped: the caller applies max(colour, 0) as the reference does.
__device__ __forceinline__ v3 shade_pixel(const ShadeParams& S, const ImageLayout& L, const ShadeImages& I, int x,
                                          int y, int64_t e, int32_t sid, v3 T, v3 sky) {
  const int c = L.channels;
  v3 color = V(0.00015f, 0.0002f, 0.00035f);  // :1302
  if (sid >= 0) {
    const v3 albedo = ld(I.albedo, e, c);
    color = albedo;
    if (S.mode == 0) {
      const v3 sun = cv(S.sun), E = cv(S.E);
      const v3 normal = vunit(ld(I.normal, e, c));
      const float ndotl = fmx(vdot(normal, sun), 0.0f);
      const v3 direct = vscale(vmul(E, T), ndotl);
      color = vmul(albedo, vadd(vdivs(direct, kPi), sky));
      if (sid == S.ocean_id && S.advanced) {
        const v3 right = cv(S.right), up = cv(S.up), fwd = cv(S.fwd);
        const v3 position = ld(I.position, e, c);
        const v3 view = vneg(vunit(vadd(vadd(vscale(right, position.x), vscale(up, position.y)),
                                        vscale(fwd, position.z))));
        const float ndotv = fmx(vdot(normal, view), 1.0e-4f);
        const v3 half_sum = vadd(view, sun);
        const v3 half_vector = vdivs(half_sum, fmx(vnorm(half_sum), 1.0e-5f));
        const float ndoth = fmx(vdot(normal, half_vector), 0.0f);
        const float vdoth = fmx(vdot(view, half_vector), 0.0f);
        const float omv = sub(1.0f, ndotv);
        const float fresnel_view = add(S.f0, mul(sub(1.0f, S.f0), mul(mul(mul(mul(omv, omv), omv), omv), omv)));
        const float omh = sub(1.0f, vdoth);
        const float fresnel_sun = add(S.f0, mul(sub(1.0f, S.f0), mul(mul(mul(mul(omh, omh), omh), omh), omh)));
        const float base_alpha = mul(S.roughness, S.roughness);
        float alpha2 = add(add(mul(base_alpha, base_alpha), I.slope_variance[e]), S.solar_slope_variance);
        alpha2 = fmn(fmx(alpha2, 1.0e-5f), 1.0f);
        const float denominator = add(mul(mul(ndoth, ndoth), sub(alpha2, 1.0f)), 1.0f);
        const float distribution = dv(alpha2, fmx(mul(mul(kPi, denominator), denominator), 1.0e-5f));
        const float effective_roughness = __fsqrt_rn(__fsqrt_rn(alpha2));
        const float er1 = add(effective_roughness, 1.0f);
        const float geometry_k = dv(mul(er1, er1), 8.0f);
        const float geometry_v = dv(ndotv, fmx(add(mul(ndotv, sub(1.0f, geometry_k)), geometry_k), 1.0e-5f));
        const float geometry_l = dv(ndotl, fmx(add(mul(ndotl, sub(1.0f, geometry_k)), geometry_k), 1.0e-5f));
        const float spec_den = fmx(mul(mul(4.0f, ndotv), ndotl), 1.0e-4f);
        v3 sun_specular = vmul(E, T);
        sun_specular = vscale(sun_specular, distribution);
        sun_specular = vscale(sun_specular, geometry_v);
        sun_specular = vscale(sun_specular, geometry_l);
        sun_specular = vscale(sun_specular, fresnel_sun);
        sun_specular = vscale(sun_specular, ndotl);
        sun_specular = vdivs(sun_specular, spec_den);
        const v3 reflected_sky = vscale(vscale(sky, fresnel_view), S.sky_strength);
        float water_depth = fmn(I.water_depth[e], S.max_depth);
        v3 seabed_albedo = ld(I.seabed_albedo, e, c);
        v3 seabed_normal = vunit(ld(I.seabed_normal, e, c));

        // refraction from air into water and the seabed behind it (:1388-1520)
        const v3 incident = vunit(position);
        const v3 normal_view = vunit(V(vdot(normal, right), vdot(normal, up), vdot(normal, fwd)));
        const float cos_incident = fmx(-vdot(incident, normal_view), 0.0f);
        const float disc = sub(1.0f, mul(mul(S.eta, S.eta), sub(1.0f, mul(cos_incident, cos_incident))));
        v3 refracted = incident;
        if (disc > 0.0f)
          refracted = vunit(vadd(vscale(incident, S.eta),
                                 vscale(normal_view, sub(mul(S.eta, cos_incident), __fsqrt_rn(disc)))));
        refracted = vunit(vadd(vscale(incident, sub(1.0f, S.strength)), vscale(refracted, S.strength)));
        const float vertical_depth = mul(water_depth, fmx(-vdot(incident, normal_view), 0.05f));
        const float refracted_distance =
            fmn(dv(vertical_depth, fmx(-vdot(refracted, normal_view), 0.05f)), mul(S.max_depth, 2.0f));
        const v3 endpoint = vadd(position, vscale(refracted, refracted_distance));
        if (endpoint.z > 0.1f && S.strength > 0.0f) {
          const float W = float(L.width), H = float(L.height);
          const float aspect = dv(W, H);
          float sx = sub(mul(add(mul(dv(endpoint.x, mul(mul(endpoint.z, S.tanfov), aspect)), 0.5f), 0.5f), W), 0.5f);
          float sy = sub(mul(add(mul(dv(endpoint.y, mul(endpoint.z, S.tanfov)), 0.5f), 0.5f), H), 0.5f);
          const float qx = float(x), qy = float(y);
          float dx = sub(sx, qx), dy = sub(sy, qy);
          const float delta_length = __fsqrt_rn(add(mul(dx, dx), mul(dy, dy)));
          if (delta_length > S.max_offset) {
            const float k = dv(S.max_offset, fmx(delta_length, 1.0e-5f));
            dx = mul(dx, k);
            dy = mul(dy, k);
            sx = add(qx, dx);
            sy = add(qy, dy);
          }
          const float fbx = floorf(sx), fby = floorf(sy);
          const int bx = int(fbx), by = int(fby);
          const float fx = sub(sx, float(bx)), fy = sub(sy, float(by));
          v3 acc_albedo = V(0.0f, 0.0f, 0.0f), acc_normal = V(0.0f, 0.0f, 0.0f), acc_position = V(0.0f, 0.0f, 0.0f);
          float acc_weight = 0.0f;
          const float near_limit = add(position.z, 0.01f), far_limit = mul(S.max_depth, 2.0f);
#pragma unroll
          for (int oy = 0; oy < 2; ++oy)
#pragma unroll
            for (int ox = 0; ox < 2; ++ox) {
              const int ix = bx + ox, iy = by + oy;
              const bool inside = ix >= 0 && ix < L.width && iy >= 0 && iy < L.height;
              const int cx = min(max(ix, 0), L.width - 1), cy = min(max(iy, 0), L.height - 1);
              const int64_t t = int64_t(cx) * L.sx + int64_t(cy) * L.sy;
              if (inside && I.terrain_surface_id[t] >= 0) {
                const v3 candidate = ld(I.terrain_position, t, c);
                const float distance = vnorm(vsub(candidate, position));
                if (candidate.z > near_limit && distance <= far_limit) {
                  const float wx = ox == 0 ? sub(1.0f, fx) : fx;
                  const float wy = oy == 0 ? sub(1.0f, fy) : fy;
                  const float weight = mul(wx, wy);
                  acc_albedo = vadd(acc_albedo, vscale(ld(I.terrain_albedo, t, c), weight));
                  acc_normal = vadd(acc_normal, vscale(ld(I.terrain_normal, t, c), weight));
                  acc_position = vadd(acc_position, vscale(candidate, weight));
                  acc_weight = add(acc_weight, weight);
                }
              }
            }
          if (acc_weight > 0.25f) {
            const float inv = dv(1.0f, acc_weight);
            seabed_albedo = vscale(acc_albedo, inv);
            seabed_normal = vunit(vscale(acc_normal, inv));
            const v3 seabed_position = vscale(acc_position, inv);
            water_depth = fmn(vnorm(vsub(seabed_position, position)), S.max_depth);
          }
        }
        // water body (:1521-1574)
        const v3 extinction = cv(S.extinction);
        const v3 tau = vscale(vneg(extinction), water_depth);
        const v3 transmission = V(expf(tau.x), expf(tau.y), expf(tau.z));
        const float seabed_ndotl = fmx(vdot(seabed_normal, sun), 0.0f);
        const v3 seabed_direct = vscale(vmul(E, T), seabed_ndotl);
        const v3 seabed = vmul(vmul(seabed_albedo, vadd(vdivs(seabed_direct, kPi), sky)), transmission);
        const v3 incident_water = vadd(sky, vdivs(direct, S.four_pi));
        const v3 water_scattering =
            vmul(vmul(incident_water, cv(S.scattering_albedo)), vsub(V(1.0f, 1.0f, 1.0f), transmission));
        const v3 water_body = vscale(vadd(seabed, water_scattering), sub(1.0f, fresnel_view));
        color = vadd(vadd(water_body, reflected_sky), sun_specular);
      }
    }
  }
  return color;
}

}  // namespace shading
}  // namespace atm
