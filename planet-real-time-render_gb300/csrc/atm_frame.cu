// atm_frame.cu - per-pixel surface lighting and the full-screen composite
// (reference atmosphere/renderer.py :1422-1472, :1474-2055) for sm_103a.
//
// The composite is the per-frame hot loop: every surface pixel integrates
// the real camera-to-G-buffer path over `aerial_horizon_raymarch_steps` warped
// base intervals, each refined into `aerial_terminator_substeps` children
// where the terminator weight is non-zero.  One thread per pixel; a warp
// covers an 8x4 pixel tile so that the data-dependent paths (sky vs surface,
// refined intervals) diverge as little as neighbouring pixels do.  The
// terminator weight reuses the disk visibility of the interval's coarse
// sample, which the reference computes twice from identical inputs.
#include <cuda_runtime.h>

#include <mutex>

#include "atm_device.cuh"
#include "atm_kernels.h"

namespace atm {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ size_t pix_offset(const ImageLayout& L, int x, int y) {
  return size_t(int64_t(x) * L.sx + int64_t(y) * L.sy);
}

// Pixel of thread: blocks of 16x16 pixels, each warp an 8x4 sub-tile.
__device__ __forceinline__ bool tile_pixel(const ImageLayout& L, int& x, int& y) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;  // 0..7
  x = blockIdx.x * 16 + (w & 1) * 8 + (lane & 7);
  y = blockIdx.y * 16 + (w >> 1) * 4 + (lane >> 3);
  return x < L.width && y < L.height;
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

// _prepare_surface_lighting :1422-1472
__global__ void __launch_bounds__(256) k_prepare_surface(DevParams P, ImageLayout L, const float* __restrict__ pos,
                                                         const int32_t* __restrict__ sid, float bottom, float cam_alt,
                                                         f3 sun, float ar, f3 right, f3 up, f3 fwd,
                                                         const float4* __restrict__ tlut,
                                                         const float4* __restrict__ mslut, float* __restrict__ out_t,
                                                         float* __restrict__ out_sky) {
  int x, y;
  if (!linear_pixel(L, x, y)) return;
  const size_t e = pix_offset(L, x, y);
  const size_t o = e * L.channels;
  Frame F = make_frame(P, tlut, mslut, bottom, ar, sun, splat(0.0f));
  f3 st = splat(1.0f), sky = splat(0.0f);
  if (sid[e] >= 0) {
    f3 vp = ld3(pos + o);
    f3 lp = (right * vp.x + up * vp.y) + fwd * vp.z;
    f3 pp = mk(lp.x, (bottom + cam_alt) + lp.y, lp.z);
    float radius = norm(pp);
    f3 radial = pp / mx(radius, 1.0f);
    float sd = norm(lp);
    f3 lr = lp / mx(sd, 1.0f);
    float h = altitude_on_ray(cam_alt, lr.y, sd, bottom);
    float sc = dot(radial, sun);
    Horizon H = horizon_at(h, bottom);
    float vis;
    st = sample_solar_t(P, F, h, sc, H, vis);
    sky = sample_ms(P, F, h, sc, H.hc);
  }
  out_t[o + 0] = st.x;
  out_t[o + 1] = st.y;
  out_t[o + 2] = st.z;
  sky = vmax(sky, 0.0f);
  out_sky[o + 0] = sky.x;
  out_sky[o + 1] = sky.y;
  out_sky[o + 2] = sky.z;
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

// _integrate_surface_scattering :1667-1755 (with :901-1032).  `start`/`end`
// are the shell-clipped interval; the caller has checked it is non-empty.
__device__ __forceinline__ f3 integrate_surface(const DevParams& P, const Frame& F, float cam_alt, f3 ray,
                                                float start, float end, uint32_t& samples) {
  const float o_y = F.bottom + cam_alt;
  const f3 origin = mk(0.0f, o_y, 0.0f);
  float sr0, sr1;
  bool sv0, sv1;
  shadow_roots(origin, ray, F.sun, F.bottom, sr0, sr1, sv0, sv1);
  const RaySource rs = make_ray_source(P, F, o_y, cam_alt, ray);
  const RayWarp rw = make_warp(-(o_y * ray.y), start, end);
  const bool roots = sv0 || sv1;
  const int n = P.limb_steps;
  const int nsub = P.substeps;
  Seg acc = {splat(0.0f), splat(1.0f)};
  float d0 = warp_at(rw, 0.0f);
  for (int i = 0; i < n; ++i) {
    float d1 = warp_at(rw, float(i + 1) / float(n));
    float vis;
    Seg coarse = source_segment<true>(P, F, rs, d0, d1, vis);
    ++samples;
    // _terminator_refinement_weight :901-966; zero unless a shadow-cylinder
    // root exists or the disk is partly hidden at the midpoint
    float w = 0.0f;
    if (roots || (vis > 0.0f && vis < 1.0f)) {
      float mid = (d0 + d1) * 0.5f;
      float iw = mx(d1 - d0, 1.0e-4f);
      float closest_root = 1.0e30f;
      if (sv0) closest_root = mn(closest_root, fabsf(mid - sr0));
      if (sv1) closest_root = mn(closest_root, fabsf(mid - sr1));
      float prox = __saturatef(2.0f - fdiv(closest_root, iw));
      prox = prox * prox * (3.0f - 2.0f * prox);
      w = mx(prox, 4.0f * vis * (1.0f - vis));
    }
    Seg interval = coarse;
    if (w > 0.0f) {
      // _integrate_adaptive_scattering_interval :998-1031
      Seg fine = {splat(0.0f), splat(1.0f)};
      float c0 = d0 + (d1 - d0) * 0.0f;
      for (int k = 0; k < nsub; ++k) {
        float c1 = d0 + (d1 - d0) * (float(k + 1) / float(nsub));
        float cvis;
        fine = seg_then(fine, source_segment<true>(P, F, rs, c0, c1, cvis));
        c0 = c1;
      }
      samples += nsub;
      interval.L = coarse.L * (1.0f - w) + fine.L * w;
      interval.T = coarse.T * (1.0f - w) + fine.T * w;
    }
    acc = seg_then(acc, interval);
    d0 = d1;
  }
  return vmax(acc.L, 0.0f);
}

// _surface_segment_transmittance :1603-1665 on an already clipped interval.
__device__ __forceinline__ f3 surface_segment_t(const DevParams& P, const Frame& F, float cam_alt, f3 ray,
                                                float start, float end) {
  const f3 origin = mk(0.0f, F.bottom + cam_alt, 0.0f);
  f3 np = origin + ray * start;
  f3 sp = origin + ray * end;
  f3 rr = -ray;
  f3 nrad = np / mx(norm(np), 1.0f);
  f3 srad = sp / mx(norm(sp), 1.0f);
  float na = altitude_on_ray(cam_alt, ray.y, start, F.bottom);
  float sa = altitude_on_ray(cam_alt, ray.y, end, F.bottom);
  f3 s2t = sample_t(P, F, sa, dot(srad, rr));
  f3 n2t = sample_t(P, F, na, dot(nrad, rr));
  return vclamp(s2t / vmax(n2t, 1.0e-6f), 0.0f, 1.0f);
}

// _camera_transmittance :1788-1825
__device__ __forceinline__ f3 camera_t(const DevParams& P, const Frame& F, float cam_alt, f3 ray) {
  float s, e;
  bool valid, ground;
  segment_from_altitude(P, cam_alt, ray.y, F.bottom, s, e, valid, ground);
  if (!valid) return splat(1.0f);
  if (ground) return splat(0.0f);
  f3 entry = mk(0.0f, F.bottom + cam_alt, 0.0f) + ray * s;
  f3 radial = entry / mx(norm(entry), 1.0f);
  float ea = altitude_on_ray(cam_alt, ray.y, s, F.bottom);
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
__device__ __forceinline__ bool surface_interval(const DevParams& P, float cam_alt, float ray_y, float bottom,
                                                 float surface_distance, float& start, float& end) {
  float on, of;
  bool oh;
  shell_roots(cam_alt, ray_y, P.top, bottom, on, of, oh);
  start = mx(on, 0.0f);
  end = mn(surface_distance, of);
  return oh && end > start;
}

__device__ __forceinline__ f3 composite_sky(const DevParams& P, const Frame& F, const CompositeScalars& A,
                                            const float4* __restrict__ svlut, f3 ray, f3 color, f3 space,
                                            float height) {
  f3 tr = camera_t(P, F, A.cam_alt, ray);
  f3 sky = sample_sky_view(P, svlut, ray, F.sun, A.sky_alt, F.bottom);
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

// COMPOSITE view (:1860-1940): the per-frame path.
__global__ void __launch_bounds__(256, 3) k_composite(DevParams P, ImageLayout L, CompositeScalars A,
                                                   const float* __restrict__ scene, const float* __restrict__ space,
                                                   const int32_t* __restrict__ sid, const float* __restrict__ pos,
                                                   const float4* __restrict__ tlut, const float4* __restrict__ mslut,
                                                   const float4* __restrict__ svlut, float* __restrict__ hdr,
                                                   unsigned long long* counter) {
  int x, y;
  const bool inside = tile_pixel(L, x, y);
  uint32_t samples = 0;
  if (inside) {
    const size_t e = pix_offset(L, x, y);
    const size_t o = e * L.channels;
    Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
    PixelRay pr = pixel_ray(L, A, x, y);
    f3 color = ld3(scene + o);
    if (sid[e] >= 0) {
      float sd = norm(ld3(pos + o));
      float start, end;
      if (surface_interval(P, A.cam_alt, pr.ray.y, A.bottom, sd, start, end)) {
        f3 scat = integrate_surface(P, F, A.cam_alt, pr.ray, start, end, samples);
        f3 tr = surface_segment_t(P, F, A.cam_alt, pr.ray, start, end);
        color = scat + color * tr;
      }
    } else {
      color = composite_sky(P, F, A, svlut, pr.ray, color, ld3(space + o), float(L.height));
    }
    color = vmax(color, 0.0f);
    hdr[o + 0] = color.x;
    hdr[o + 1] = color.y;
    hdr[o + 2] = color.z;
  }
  warp_count(samples, counter);
}

// _sample_aerial_field :1527-1571 (volume stored [z][y][x])
__device__ __forceinline__ f3 sample_aerial_field(const DevParams& P, const float4* __restrict__ ap, float su,
                                                  float sv, float df) {
  float x = clampf(su * float(P.ap_w) - 0.5f, 0.0f, float(P.ap_w - 1));
  float y = clampf(sv * float(P.ap_h) - 0.5f, 0.0f, float(P.ap_h - 1));
  float z = clampf(df, 0.0f, 1.0f) * float(P.ap_d - 1);
  int x0 = int(floorf(x)), y0 = int(floorf(y)), z0 = int(floorf(z));
  int x1 = min(x0 + 1, P.ap_w - 1), y1 = min(y0 + 1, P.ap_h - 1), z1 = min(z0 + 1, P.ap_d - 1);
  float fx = x - float(x0), fy = y - float(y0), fz = z - float(z0);
  auto at = [&](int xi, int yi, int zi) { return from4(__ldg(ap + (size_t(zi) * P.ap_h + yi) * P.ap_w + xi)); };
  f3 a = at(x0, y0, z0) * (1.0f - fx) + at(x1, y0, z0) * fx;
  f3 b = at(x0, y1, z0) * (1.0f - fx) + at(x1, y1, z0) * fx;
  f3 c = at(x0, y0, z1) * (1.0f - fx) + at(x1, y0, z1) * fx;
  f3 d = at(x0, y1, z1) * (1.0f - fx) + at(x1, y1, z1) * fx;
  f3 lo = a * (1.0f - fy) + b * fy;
  f3 hi = c * (1.0f - fy) + d * fy;
  return lo * (1.0f - fz) + hi * fz;
}

// Diagnostic views (:1941-2052); not on the per-frame path.
__global__ void __launch_bounds__(256, 3) k_composite_views(DevParams P, ImageLayout L, CompositeScalars A,
                                                         const float* __restrict__ scene,
                                                         const float* __restrict__ space,
                                                         const int32_t* __restrict__ sid,
                                                         const float* __restrict__ pos,
                                                         const float4* __restrict__ tlut,
                                                         const float4* __restrict__ mslut,
                                                         const float4* __restrict__ svlut,
                                                         const float4* __restrict__ aplut, float* __restrict__ hdr,
                                                         unsigned long long* counter) {
  int x, y;
  const bool inside = tile_pixel(L, x, y);
  uint32_t samples = 0;
  if (inside) {
    const size_t e = pix_offset(L, x, y);
    const size_t o = e * L.channels;
    Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
    PixelRay pr = pixel_ray(L, A, x, y);
    const bool surface = sid[e] >= 0;
    f3 color = ld3(scene + o);
    switch (A.view) {
      case ATM_VIEW_SKY_VIEW:
        color = sample_sky_view(P, svlut, pr.ray, F.sun, A.sky_alt, A.bottom);
        break;
      case ATM_VIEW_CAMERA_TRANSMITTANCE:
        color = camera_t(P, F, A.cam_alt, pr.ray);
        break;
      case ATM_VIEW_TRANSMITTANCE_LUT: {
        int lx = min(int(pr.su * float(P.t_w)), P.t_w - 1);
        int ly = min(int(pr.sv * float(P.t_h)), P.t_h - 1);
        color = from4(tlut[ly * P.t_w + lx]);
        break;
      }
      case ATM_VIEW_MULTI_SCATTERING_LUT: {
        int lx = min(int(pr.su * float(P.ms_w)), P.ms_w - 1);
        int ly = min(int(pr.sv * float(P.ms_h)), P.ms_h - 1);
        color = from4(mslut[ly * P.ms_w + lx]);
        break;
      }
      case ATM_VIEW_AERIAL_SCATTERING:
      case ATM_VIEW_AERIAL_DIRECT_ONLY: {
        color = splat(0.0f);
        float start, end;
        if (surface && surface_interval(P, A.cam_alt, pr.ray.y, A.bottom, norm(ld3(pos + o)), start, end))
          color = integrate_surface(P, F, A.cam_alt, pr.ray, start, end, samples);
        break;
      }
      case ATM_VIEW_AERIAL_FROXEL_ONLY: {
        color = splat(0.0f);
        if (surface) {
          float s, e2;
          bool valid;
          aerial_prefix(P, A.cam_alt, pr.ray.y, A.bottom, s, e2, valid);
          float df = 0.0f;
          if (valid) df = clampf((norm(ld3(pos + o)) - s) / mx(e2 - s, 1.0f), 0.0f, 1.0f);
          color = sample_aerial_field(P, aplut, pr.su, pr.sv, df);
        }
        break;
      }
      case ATM_VIEW_AERIAL_BLEND_WEIGHT:
        color = splat(surface ? 1.0f : 0.0f);
        break;
      case ATM_VIEW_AERIAL_TRANSMITTANCE: {
        color = splat(0.0f);
        if (surface) {
          float start, end;
          color = splat(1.0f);
          if (surface_interval(P, A.cam_alt, pr.ray.y, A.bottom, norm(ld3(pos + o)), start, end))
            color = surface_segment_t(P, F, A.cam_alt, pr.ray, start, end);
        }
        break;
      }
      default:  // SURFACE_MASK and any other value
        color = splat(surface ? 1.0f : 0.0f);
        break;
    }
    color = vmax(color, 0.0f);
    hdr[o + 0] = color.x;
    hdr[o + 1] = color.y;
    hdr[o + 2] = color.z;
  }
  warp_count(samples, counter);
}

inline f3 host3(const float* v) { return {v[0], v[1], v[2]}; }

inline dim3 tile_grid(const ImageLayout& L) { return dim3((L.width + 15) / 16, (L.height + 15) / 16); }

}  // namespace

cudaError_t launch_prepare_surface(const DevParams& P, const ImageLayout& L, const float* pos, const int32_t* sid,
                                   float bottom, float cam_alt, const float sun[3], float ar, const float right[3],
                                   const float up[3], const float fwd[3], const float4* tlut, const float4* mslut,
                                   float* out_sun_t, float* out_sky, cudaStream_t s) {
  const unsigned blocks = unsigned((static_cast<long long>(L.width) * L.height + 255) / 256);
  k_prepare_surface<<<blocks, 256, 0, s>>>(P, L, pos, sid, bottom, cam_alt, host3(sun), ar, host3(right),
                                                 host3(up), host3(fwd), tlut, mslut, out_sun_t, out_sky);
  return cudaGetLastError();
}

cudaError_t launch_composite(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                             const float* scene, const float* space, const int32_t* sid, const float* pos,
                             const float4* tlut, const float4* mslut, const float4* svlut, const float4* aplut,
                             float* hdr, unsigned long long* sample_counter, cudaStream_t s) {
  if (A.view == ATM_VIEW_COMPOSITE)
    k_composite<<<tile_grid(L), 256, 0, s>>>(P, L, A, scene, space, sid, pos, tlut, mslut, svlut, hdr,
                                             sample_counter);
  else
    k_composite_views<<<tile_grid(L), 256, 0, s>>>(P, L, A, scene, space, sid, pos, tlut, mslut, svlut, aplut, hdr,
                                                   sample_counter);
  return cudaGetLastError();
}


// ---- composite that allocates nothing -------------------------------------
// Scratch of atm_composite_noalloc: one radiance-sample count per 16x16
// pixel tile.  It lives in this file-scope device array, so a caller that
// may not allocate device memory can still get the sample count; every GPU
// that loads the library holds these 256 KB until the process exits.  Host
// code must not use the symbol as an address: noalloc_tile_scratch() looks
// the device address up with cudaGetSymbolAddress.
constexpr int kNoAllocMaxTiles = 1 << 16;  // 65,536 tiles = 16.7 Mpx
static __device__ __align__(256) uint32_t g_noalloc_tile_samples[kNoAllocMaxTiles];

namespace {

// COMPOSITE view of k_composite; the block's sample count goes to its tile
// slot instead of an atomic counter (every launched block writes its slot).
__global__ void __launch_bounds__(256, 3) k_composite_tiles(DevParams P, ImageLayout L, CompositeScalars A,
                                                         const float* __restrict__ scene,
                                                         const float* __restrict__ space,
                                                         const int32_t* __restrict__ sid,
                                                         const float* __restrict__ pos,
                                                         const float4* __restrict__ tlut,
                                                         const float4* __restrict__ mslut,
                                                         const float4* __restrict__ svlut, float* __restrict__ hdr,
                                                         uint32_t* __restrict__ tile_samples) {
  __shared__ uint32_t s_warp[8];
  int x, y;
  const bool inside = tile_pixel(L, x, y);
  uint32_t samples = 0;
  if (inside) {
    const size_t e = pix_offset(L, x, y);
    const size_t o = e * L.channels;
    Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
    PixelRay pr = pixel_ray(L, A, x, y);
    f3 color = ld3(scene + o);
    if (sid[e] >= 0) {
      float sd = norm(ld3(pos + o));
      float start, end;
      if (surface_interval(P, A.cam_alt, pr.ray.y, A.bottom, sd, start, end)) {
        f3 scat = integrate_surface(P, F, A.cam_alt, pr.ray, start, end, samples);
        f3 tr = surface_segment_t(P, F, A.cam_alt, pr.ray, start, end);
        color = scat + color * tr;
      }
    } else {
      color = composite_sky(P, F, A, svlut, pr.ray, color, ld3(space + o), float(L.height));
    }
    color = vmax(color, 0.0f);
    hdr[o + 0] = color.x;
    hdr[o + 1] = color.y;
    hdr[o + 2] = color.z;
  }
  __syncwarp();
#pragma unroll
  for (int k = 16; k > 0; k >>= 1) samples += __shfl_xor_sync(kFull, samples, k);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = samples;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t total = 0;
    for (int w = 0; w < 8; ++w) total += s_warp[w];
    tile_samples[blockIdx.y * gridDim.x + blockIdx.x] = total;
  }
}

// Sum of n tile counts into *out (one block, fixed order: deterministic).
__global__ void __launch_bounds__(1024) k_sum_tiles(const uint32_t* __restrict__ tiles, int n,
                                                    unsigned long long* __restrict__ out) {
  __shared__ unsigned long long s[1024];
  unsigned long long acc = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += tiles[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

std::mutex g_noalloc_mutex;
uint32_t* g_noalloc_address[kMaxDevices] = {};

}  // namespace

int noalloc_max_tiles() { return kNoAllocMaxTiles; }

cudaError_t noalloc_tile_scratch(uint32_t** out) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return e;
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_address[device] == nullptr) {
    void* address = nullptr;
    e = cudaGetSymbolAddress(&address, g_noalloc_tile_samples);  // with `device` current
    if (e != cudaSuccess) return e;
    g_noalloc_address[device] = static_cast<uint32_t*>(address);
  }
  *out = g_noalloc_address[device];
  return cudaSuccess;
}

cudaError_t launch_composite_noalloc(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                                     const float* scene, const float* space, const int32_t* sid, const float* pos,
                                     const float4* tlut, const float4* mslut, const float4* svlut, float* hdr,
                                     uint32_t* tile_scratch, unsigned long long* samples_out, cudaStream_t s) {
  const dim3 grid = tile_grid(L);
  k_composite_tiles<<<grid, 256, 0, s>>>(P, L, A, scene, space, sid, pos, tlut, mslut, svlut, hdr, tile_scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || samples_out == nullptr) return e;
  k_sum_tiles<<<1, 1024, 0, s>>>(tile_scratch, int(grid.x * grid.y), samples_out);
  return cudaGetLastError();
}

}  // namespace atm
