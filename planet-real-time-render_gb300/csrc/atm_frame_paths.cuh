// atm_frame_paths.cuh - per-pixel paths of the composite (reference
// atmosphere/renderer.py :1474-1940): pixel rays, the G-buffer-bounded limb
// integrator, the transmittance ratio, camera transmittance and the sky
// branch.  Shared by the plain composite and the surrogate composite.
#pragma once

#include "atm_device.cuh"
#include "atm_kernels.h"
#include "atm_shade.cuh"

namespace atm {

__device__ __forceinline__ size_t pix_offset(const ImageLayout& L, int x, int y) {
  return size_t(int64_t(x) * L.sx + int64_t(y) * L.sy);
}

// Pixel of thread in the 16x16 pixel block (bx, by): each warp an 8x4 sub-tile.
__device__ __forceinline__ bool tile_pixel_at(const ImageLayout& L, int bx, int by, int& x, int& y) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;  // 0..7
  x = bx * 16 + (w & 1) * 8 + (lane & 7);
  y = by * 16 + (w >> 1) * 4 + (lane >> 3);
  return x < L.width && y < L.height;
}
__device__ __forceinline__ bool tile_pixel(const ImageLayout& L, int& x, int& y) {
  return tile_pixel_at(L, blockIdx.x, blockIdx.y, x, y);
}

// Pixel of a thread for memory-bound per-pixel kernels: consecutive threads
// take consecutive elements along the image's contiguous dimension.
__device__ __forceinline__ bool linear_pixel(const ImageLayout& L, int& x, int& y) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)L.width * L.height) return false;
  if (L.sy <= L.sx) {  // y contiguous: the reference's (W, H, 3) layout
    x = int(i / L.height);
    y = int(i % L.height);
  } else {
    y = int(i / L.width);
    x = int(i % L.width);
  }
  return true;
}

struct PixelRay {
  f3 ray;
  float su, sv;
};
__device__ __forceinline__ PixelRay pixel_ray(const ImageLayout& L, const CompositeScalars& A, int x, int y) {
  PixelRay r;
  const float aspect = float(L.width) / float(L.height);
  r.su = (float(x) + 0.5f) / float(L.width);
  r.sv = (float(y) + 0.5f) / float(L.height);
  float sx = (r.su * 2.0f - 1.0f) * aspect;
  float sy = r.sv * 2.0f - 1.0f;
  f3 rv = (arr3(A.right) * sx + arr3(A.up) * sy) + arr3(A.fwd) / A.tanfov;
  r.ray = rv * (1.0f / norm(rv));
  return r;
}

// _solar_shadow_roots :685-726
__device__ __forceinline__ void shadow_roots(f3 o, f3 d, f3 sun, float bottom, float& r0, float& r1, bool& v0,
                                             bool& v1) {
  f3 op = o - sun * dot(o, sun);
  f3 rp = d - sun * dot(d, sun);
  float quad = dot(rp, rp);
  float hl = dot(op, rp);
  float pl = norm(op);
  float c = (pl - bottom) * (pl + bottom);
  r0 = 0.0f;
  r1 = 0.0f;
  v0 = false;
  v1 = false;
  float disc = hl * hl - quad * c;
  if (quad > 1.0e-8f && disc >= 0.0f) {
    float sr = sqrtf(mx(disc, 0.0f));
    r0 = (-hl - sr) / quad;
    r1 = (-hl + sr) / quad;
    v0 = dot(o + d * r0, sun) < 0.0f;
    v1 = dot(o + d * r1, sun) < 0.0f;
  }
}
// The same roots in FP64 for a camera above the shell, whose distance to the
// shadow cylinder's axis makes hl^2 and quad c cancel in float.  The origin
// is (0, o_y, 0) with o_y = bottom + h0 formed in double.
__device__ __forceinline__ void shadow_roots_far(float h0, f3 df, f3 sf, float bottom, float& r0, float& r1,
                                                 bool& v0, bool& v1) {
  const double oy = double(bottom) + double(h0), b = bottom;
  const double dx = df.x, dy = df.y, dz = df.z, sx = sf.x, sy = sf.y, sz = sf.z;
  const double os = oy * sy, ds = dx * sx + dy * sy + dz * sz;
  const double opx = -sx * os, opy = oy - sy * os, opz = -sz * os;
  const double rpx = dx - sx * ds, rpy = dy - sy * ds, rpz = dz - sz * ds;
  const double quad = rpx * rpx + rpy * rpy + rpz * rpz;
  const double hl = opx * rpx + opy * rpy + opz * rpz;
  const double pl = sqrt(opx * opx + opy * opy + opz * opz);
  const double c = (pl - b) * (pl + b);
  const double disc = hl * hl - quad * c;
  r0 = 0.0f;
  r1 = 0.0f;
  v0 = false;
  v1 = false;
  if (quad > 1.0e-8 && disc >= 0.0) {
    const double sr = sqrt(disc);
    const double t0 = (-hl - sr) / quad, t1 = (-hl + sr) / quad;
    r0 = float(t0);
    r1 = float(t1);
    v0 = os + t0 * ds < 0.0;
    v1 = os + t1 * ds < 0.0;
  }
}

// Geometry of a camera ray (sine from the horizontal components).
__device__ __forceinline__ RayGeom camera_ray_geom(const DevParams& P, float bottom, float h0, f3 ray);

// _prepare_surface_lighting :1422-1472 for one surface pixel: the finite-disk
// sun transmittance `st` and the multi-scattering sky radiance `sky`
// (clamped at 0) at its view-space position vp.
__device__ __forceinline__ void surface_lighting(const DevParams& P, const Frame& F, float cam_alt, f3 right, f3 up,
                                                 f3 fwd, f3 vp, f3& st, f3& sky) {
  const float bottom = F.bottom;
  const f3 sun = F.sun;
  f3 lp = (right * vp.x + up * vp.y) + fwd * vp.z;
  f3 pp = mk(lp.x, (bottom + cam_alt) + lp.y, lp.z);
  float radius = norm(pp);
  f3 radial = pp / mx(radius, 1.0f);
  float sd = norm(lp);
  f3 lr = lp / mx(sd, 1.0f);
  float h, sc;
  if (!far_camera(P, bottom, cam_alt)) {
    h = altitude_on_ray(cam_alt, lr.y, sd, bottom);
    sc = dot(radial, sun);
  } else {  // camera above the shell: pivot at the closest approach (RayGeom)
    const RayGeom G = camera_ray_geom(P, bottom, cam_alt, lr);
    h = altitude_at(G, sd, bottom);
    // p . sun = o . sun + t_c lr . sun + (t - t_c) lr . sun, the first two in
    // FP64 (the point's own coordinates cancel like its altitude)
    const double s0 = (double(bottom) + double(cam_alt)) * double(sun.y) +
                      double(G.tc) * (double(lr.x) * sun.x + double(lr.y) * sun.y + double(lr.z) * sun.z);
    sc = (float(s0) + (sd - G.tc) * dot(lr, sun)) * frcp(bottom + h);
  }
  Horizon H = horizon_at(h, bottom);
  float vis;
  st = sample_solar_t(P, F, h, sc, H, vis);
  sky = vmax(sample_ms(P, F, h, sc, H.hc), 0.0f);
}

__device__ __forceinline__ RayGeom camera_ray_geom(const DevParams& P, float bottom, float h0, f3 ray) {
  return ray_geom(P, bottom, h0, ray.y, sqrtf(ray.x * ray.x + ray.z * ray.z));
}

// Per-ray state of the limb integrator (_integrate_surface_scattering
// :1667-1755): shadow-cylinder roots, the ray's source terms and the
// distribution of its base intervals over [start, end].
struct SurfaceMarch {
  RaySource rs;
  RayWarp rw;
  float sr0, sr1;
  bool sv0, sv1;
};
__device__ __forceinline__ SurfaceMarch make_surface_march(const DevParams& P, const Frame& F, const RayGeom& G, f3 ray,
                                                           float start, float end) {
  SurfaceMarch M;
  if (G.far)
    shadow_roots_far(G.h0, ray, F.sun, F.bottom, M.sr0, M.sr1, M.sv0, M.sv1);
  else
    shadow_roots(mk(0.0f, F.bottom + G.h0, 0.0f), ray, F.sun, F.bottom, M.sr0, M.sr1, M.sv0, M.sv1);
  M.rs = make_ray_source(P, F, G, ray);
  M.rw = make_warp(G.tc, start, end);
  return M;
}
// One base interval [d0, d1] with its terminator refinement (:901-1031).
__device__ __forceinline__ Seg surface_interval_seg(const DevParams& P, const Frame& F, const SurfaceMarch& M, float d0,
                                                    float d1, uint32_t& samples) {
  float vis;
  Seg coarse = source_segment<true>(P, F, M.rs, d0, d1, vis);
  ++samples;
  // _terminator_refinement_weight :901-966; zero unless a shadow-cylinder
  // root exists or the disk is partly hidden at the midpoint
  float w = 0.0f;
  if ((M.sv0 || M.sv1) || (vis > 0.0f && vis < 1.0f)) {
    float mid = (d0 + d1) * 0.5f;
    float iw = mx(d1 - d0, 1.0e-4f);
    float closest_root = 1.0e30f;
    if (M.sv0) closest_root = mn(closest_root, fabsf(mid - M.sr0));
    if (M.sv1) closest_root = mn(closest_root, fabsf(mid - M.sr1));
    float prox = __saturatef(2.0f - fdiv(closest_root, iw));
    prox = prox * prox * (3.0f - 2.0f * prox);
    w = mx(prox, 4.0f * vis * (1.0f - vis));
  }
  Seg interval = coarse;
  if (w > 0.0f) {
    // _integrate_adaptive_scattering_interval :998-1031
    const int nsub = P.substeps;
    Seg fine = {splat(0.0f), splat(1.0f)};
    float c0 = d0 + (d1 - d0) * 0.0f;
    for (int k = 0; k < nsub; ++k) {
      float c1 = d0 + (d1 - d0) * (float(k + 1) / float(nsub));
      float cvis;
      fine = seg_then(fine, source_segment<true>(P, F, M.rs, c0, c1, cvis));
      c0 = c1;
    }
    samples += nsub;
    interval.L = coarse.L * (1.0f - w) + fine.L * w;
    interval.T = coarse.T * (1.0f - w) + fine.T * w;
  }
  return interval;
}

// _integrate_surface_scattering :1667-1755 (with :901-1032).  `start`/`end`
// are the shell-clipped interval; the caller has checked it is non-empty.
__device__ __forceinline__ f3 integrate_surface(const DevParams& P, const Frame& F, const RayGeom& G, f3 ray,
                                                float start, float end, uint32_t& samples) {
  const SurfaceMarch M = make_surface_march(P, F, G, ray, start, end);
  const int n = P.limb_steps;
  Seg acc = {splat(0.0f), splat(1.0f)};
  float d0 = warp_at(M.rw, 0.0f);
  for (int i = 0; i < n; ++i) {
    float d1 = warp_at(M.rw, float(i + 1) / float(n));
    acc = seg_then(acc, surface_interval_seg(P, F, M, d0, d1, samples));
    d0 = d1;
  }
  return vmax(acc.L, 0.0f);
}

// _surface_segment_transmittance :1603-1665 on an already clipped interval.
__device__ __forceinline__ f3 surface_segment_t(const DevParams& P, const Frame& F, const RayGeom& G, f3 ray,
                                                float start, float end) {
  f3 s2t, n2t;
  if (!G.far) {
    const float cam_alt = G.h0;
    const f3 origin = mk(0.0f, F.bottom + cam_alt, 0.0f);
    f3 np = origin + ray * start;
    f3 sp = origin + ray * end;
    f3 rr = -ray;
    f3 nrad = np / mx(norm(np), 1.0f);
    f3 srad = sp / mx(norm(sp), 1.0f);
    float na = altitude_on_ray(cam_alt, ray.y, start, F.bottom);
    float sa = altitude_on_ray(cam_alt, ray.y, end, F.bottom);
    s2t = sample_t(P, F, sa, dot(srad, rr));
    n2t = sample_t(P, F, na, dot(nrad, rr));
  } else {  // radial . (-ray) = -(t - t_c) / r
    const float na = altitude_at(G, start, F.bottom), sa = altitude_at(G, end, F.bottom);
    s2t = sample_t(P, F, sa, -vertical_cosine_at(G, end, F.bottom + sa));
    n2t = sample_t(P, F, na, -vertical_cosine_at(G, start, F.bottom + na));
  }
  return vclamp(s2t / vmax(n2t, 1.0e-6f), 0.0f, 1.0f);
}

// _camera_transmittance :1788-1825
__device__ __forceinline__ f3 camera_t(const DevParams& P, const Frame& F, const RayGeom& G, f3 ray) {
  float s, e;
  bool valid, ground;
  segment_of(P, G, F.bottom, s, e, valid, ground);
  if (!valid) return splat(1.0f);
  if (ground) return splat(0.0f);
  if (G.far) {
    const float ea = altitude_at(G, s, F.bottom);
    return sample_t(P, F, ea, vertical_cosine_at(G, s, F.bottom + ea));
  }
  f3 entry = mk(0.0f, F.bottom + G.h0, 0.0f) + ray * s;
  f3 radial = entry / mx(norm(entry), 1.0f);
  float ea = altitude_on_ray(G.h0, ray.y, s, F.bottom);
  return sample_t(P, F, ea, dot(radial, ray));
}

// _sample_sky_view :1474-1525
__device__ __forceinline__ f3 sample_sky_view(const DevParams& P, const float4* __restrict__ svlut, f3 ray, f3 sun,
                                              float sky_alt, float bottom) {
  float zen = acosf(clampf(ray.y, -1.0f, 1.0f));
  float vl = sqrtf(ray.x * ray.x + ray.z * ray.z);
  float sl = sqrtf(sun.x * sun.x + sun.z * sun.z);
  float ra = 0.0f;
  if (vl > 1.0e-6f && sl > 1.0e-6f) ra = acosf(clampf((ray.x * sun.x + ray.z * sun.z) / (vl * sl), -1.0f, 1.0f));
  float u = ra / kPiF;
  float v = sky_zenith_to_v(zen, sky_horizon_zenith(sky_alt, bottom));
  return bilinear(svlut, P.sv_w, P.sv_h, u, v);
}

// Shell clip shared by the scattering integral and the transmittance ratio.
__device__ __forceinline__ bool surface_interval(const DevParams& P, const RayGeom& G, float bottom,
                                                 float surface_distance, float& start, float& end) {
  float on, of;
  bool oh;
  shell_roots_g(G, P.top, bottom, on, of, oh);
  start = mx(on, 0.0f);
  end = mn(surface_distance, of);
  return oh && end > start;
}

// Sky branch of the COMPOSITE view (:1883-1940) given the sky radiance.
__device__ __forceinline__ f3 composite_sky_with(const DevParams& P, const Frame& F, const CompositeScalars& A, f3 sky,
                                                 f3 ray, f3 color, f3 space, float height) {
  f3 tr = camera_t(P, F, camera_ray_geom(P, F.bottom, A.cam_alt, ray), ray);
  f3 star = space * tr;
  const f3 lw = mk(0.2126f, 0.7152f, 0.0722f);
  float contrast = dot(star, lw) / mx(dot(sky, lw), 1.0e-5f);
  float vis = clampf((contrast - A.star_start) / mx(A.star_end - A.star_start, 1.0e-5f), 0.0f, 1.0f);
  vis = vis * vis * (3.0f - 2.0f * vis);
  color = (sky + color * tr) + star * vis;
  float ad = acosf(clampf(dot(ray, F.sun), -1.0f, 1.0f));
  float pf = atan2f(A.tanfov * 1.41421356f / height, 1.0f);
  float cov = clampf((F.ar + pf - ad) / mx(2.0f * pf, 1.0e-8f), 0.0f, 1.0f);
  cov = cov * cov * (3.0f - 2.0f * cov);
  return color + arr3(A.disk) * tr * cov;
}

__device__ __forceinline__ f3 composite_sky(const DevParams& P, const Frame& F, const CompositeScalars& A,
                                            const float4* __restrict__ svlut, f3 ray, f3 color, f3 space,
                                            float height) {
  return composite_sky_with(P, F, A, sample_sky_view(P, svlut, ray, F.sun, A.sky_alt, F.bottom), ray, color, space,
                            height);
}


// The surface colour the composite reads as scene_hdr, formed in registers:
// the pixel's surface lighting (_prepare_surface_lighting) feeding its
// surface shading (_shade_surface), clamped at 0 as the shading writes it.
// `pos` and `sid` are the G-buffer the shading images I also hold.
__device__ __forceinline__ f3 shaded_scene(const DevParams& P, const Frame& F, const CompositeScalars& A,
                                           const ShadeParams& S, const ImageLayout& L, const ShadeImages& I, int x,
                                           int y, size_t e, int32_t sid) {
  shading::v3 T = {0.0f, 0.0f, 0.0f}, sky = {0.0f, 0.0f, 0.0f};
  if (sid >= 0 && S.mode == 0) {
    f3 st, sk;
    surface_lighting(P, F, A.cam_alt, arr3(A.right), arr3(A.up), arr3(A.fwd), ld3(I.position + e * L.channels), st,
                     sk);
    T = {st.x, st.y, st.z};
    sky = {sk.x, sk.y, sk.z};
  }
  const shading::v3 c = shading::vmax0(shading::shade_pixel(S, L, I, x, y, int64_t(e), sid, T, sky));
  return mk(c.x, c.y, c.z);
}

}  // namespace atm