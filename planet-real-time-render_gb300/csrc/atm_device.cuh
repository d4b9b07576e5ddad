// atm_device.cuh - device math of the spherical-atmosphere model (sm_103a).
//
// FP32 formulation of the reference's Taichi functions in
// src/planet_renderer/atmosphere/renderer.py (line numbers below).  The
// arithmetic follows the reference expression by expression so results agree
// with it to float rounding; where the reference evaluates the same quantity
// twice with identical inputs (density in extinction and source; horizon and
// sun zenith in disk visibility and representative zenith; a base
// interval's upper boundary and the next one's lower boundary; the
// terminator weight's midpoint visibility and the coarse sample's) it is
// evaluated once here - same inputs, same operations, same value.
//
// LUT storage: float4 texels (rgb + pad), row-major, index y * width + x;
// the aerial volume is [z][y][x].  Reads go through the read-only path.
#pragma once

#include <cstdint>

namespace atm {

constexpr float kPiF = 3.14159265358979323846f;  // f32(math.pi), renderer.py:12
constexpr float kLargeF = 1.0e30f;               // _LARGE_DISTANCE, :13

// Parameters rounded to float exactly where the Taichi trace rounds them
// (Python constants fold in double, then meet f32 values).
struct DevParams {
  float top;                   // top_altitude_m
  float beta_r[3];             // Rayleigh scattering
  float beta_ms[3];            // Mie scattering
  float beta_me[3];            // Mie extinction
  float beta_o[3];             // ozone absorption
  float albedo[3];             // ground albedo
  float h_r, h_m;              // scale heights
  float oz_peak, oz_half;      // ozone tent
  float mie_c1, mie_c2;        // f32(1+g^2), f32(2g)
  float mie_k1, mie_k2;        // f32(3(1-g^2)), f32(8 pi (2+g^2))
  float ray_k;                 // f32(16 pi)
  float inv_h_r, inv_h_m, inv_oz_half, inv_top;  // f32 reciprocals of the above
  int t_w, t_h, ms_w, ms_h, sv_w, sv_h, ap_w, ap_h, ap_d;
  int t_steps, ms_dirs, ms_steps, sv_steps, ap_steps, limb_steps, substeps;
};

struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 splat(float s) { return {s, s, s}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ f3 operator/(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float norm(f3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float mx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float mn(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return mn(mx(x, lo), hi); }
__device__ __forceinline__ f3 vmax(f3 a, float s) { return {mx(a.x, s), mx(a.y, s), mx(a.z, s)}; }
__device__ __forceinline__ f3 vmin(f3 a, float s) { return {mn(a.x, s), mn(a.y, s), mn(a.z, s)}; }
__device__ __forceinline__ f3 vclamp(f3 a, float lo, float hi) { return vmin(vmax(a, lo), hi); }
__device__ __forceinline__ f3 vexp(f3 a) { return {expf(a.x), expf(a.y), expf(a.z)}; }
__device__ __forceinline__ f3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ f3 from4(float4 v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ float4 to4(f3 v) { return make_float4(v.x, v.y, v.z, 0.0f); }
__device__ __forceinline__ f3 arr3(const float (&a)[3]) { return {a[0], a[1], a[2]}; }

// Fast forms used where no Earth-scale cancellation follows: division with
// at most 2 ulp error (div.approx) and square root with at most 1 ulp
// (sqrt.approx).  Differences ~1e-7 relative against the reference's IEEE
// operations, far below the 1e-3 parity tolerance.  Subtractions of two
// Earth-scale quantities keep IEEE sqrtf / division (see callers).
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float frcp(float b) { return __fdividef(1.0f, b); }
__device__ __forceinline__ float fsqrt(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float fnorm(f3 a) { return fsqrt(dot(a, a)); }

// Adds a per-lane count into a device counter: one atomic per warp.  Every
// lane of the warp must call it (no lane may have exited before).
__device__ __forceinline__ void warp_count(uint32_t n, unsigned long long* counter) {
  __syncwarp();
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if (counter != nullptr && (threadIdx.x & 31) == 0 && n) atomicAdd(counter, (unsigned long long)n);
}

// Composition of two consecutive ray segments: (L1,T1) then (L2,T2).
struct Seg {
  f3 L, T;
};
__device__ __forceinline__ Seg seg_then(Seg a, Seg b) { return {a.L + a.T * b.L, a.T * b.T}; }

// ---- density and coefficients (:168-209) ----------------------------------
struct Density {
  float r, m, o;
};
__device__ __forceinline__ Density density(const DevParams& P, float h) {
  Density d{0.0f, 0.0f, 0.0f};
  if (0.0f <= h && h <= P.top) {
    d.r = __expf(-h * P.inv_h_r);
    d.m = __expf(-h * P.inv_h_m);
    d.o = mx(1.0f - fabsf(h - P.oz_peak) * P.inv_oz_half, 0.0f);
  }
  return d;
}
__device__ __forceinline__ f3 extinction_of(const DevParams& P, Density d) {
  return (arr3(P.beta_r) * d.r + arr3(P.beta_me) * d.m) + arr3(P.beta_o) * d.o;
}
__device__ __forceinline__ f3 scattering_of(const DevParams& P, Density d) {
  return arr3(P.beta_r) * d.r + arr3(P.beta_ms) * d.m;
}

// ---- shells and intervals (:211-408) ---------------------------------------
__device__ __forceinline__ void sphere_roots(f3 o, f3 d, float radius, float& nearv, float& farv, bool& hit) {
  float projected = dot(o, d);
  float perpendicular = norm(o - d * projected);
  float clearance = radius - perpendicular;
  hit = clearance >= 0.0f;
  nearv = kLargeF;
  farv = -kLargeF;
  if (hit) {
    float root = sqrtf(mx(mx(clearance, 0.0f) * (radius + perpendicular), 0.0f));
    nearv = -projected - root;
    farv = -projected + root;
  }
}
__device__ __forceinline__ float shell_rho(float h, float bottom) {
  float a = mx(h, 0.0f);
  return fsqrt(a * (2.0f * bottom + a));
}
// Cancellation-free form: the altitude never subtracts two Earth-scale radii.
__device__ __forceinline__ float altitude_on_ray(float h0, float cosv, float t, float bottom) {
  float a = mx(h0, 0.0f);
  float orad = bottom + a;
  float delta = (a * (2.0f * bottom + a) + 2.0f * orad * cosv * t) + t * t;
  float len = fsqrt(mx(bottom * bottom + delta, 0.0f));
  return fdiv(delta, mx(len + bottom, 1.0f));
}
__device__ __forceinline__ void shell_roots(float h0, float cosv, float shell, float bottom, float& nearv,
                                            float& farv, bool& hit) {
  float orad = bottom + h0;
  float hl = orad * cosv;
  float c = (h0 - shell) * ((2.0f * bottom + h0) + shell);
  float disc = hl * hl - c;
  hit = disc >= 0.0f;
  nearv = kLargeF;
  farv = -kLargeF;
  if (hit) {
    float root = sqrtf(mx(disc, 0.0f));
    float sign = hl < 0.0f ? -1.0f : 1.0f;
    float q = -hl - sign * root;
    float r0 = -hl - root;
    float r1 = -hl + root;
    if (fabsf(q) > 1.0e-12f) {
      r0 = q;
      r1 = fdiv(c, q);
    }
    nearv = mn(r0, r1);
    farv = mx(r0, r1);
  }
}
__device__ __forceinline__ void segment_from_altitude(const DevParams& P, float h, float cosv, float bottom,
                                                      float& start, float& end, bool& valid, bool& ground) {
  float on, of;
  bool oh;
  shell_roots(h, cosv, P.top, bottom, on, of, oh);
  start = mx(on, 0.0f);
  end = of;
  valid = oh && end > start;
  ground = false;
  float gn, gf;
  bool gh;
  shell_roots(h, cosv, 0.0f, bottom, gn, gf, gh);
  if (valid && gh) {
    float gd = kLargeF;
    if (gn > start + 1.0e-3f)
      gd = gn;
    else if (gf > start + 1.0e-3f)
      gd = gf;
    if (gd < end) {
      end = gd;
      ground = true;
    }
  }
}
__device__ __forceinline__ void segment_vec(const DevParams& P, f3 o, f3 d, float bottom, float& start, float& end,
                                            bool& valid, bool& ground) {
  float on, of;
  bool oh;
  sphere_roots(o, d, bottom + P.top, on, of, oh);
  start = mx(on, 0.0f);
  end = of;
  valid = oh && end > start;
  ground = false;
  float gn, gf;
  bool gh;
  sphere_roots(o, d, bottom, gn, gf, gh);
  if (valid && gh) {
    float gd = kLargeF;
    float eps = mx(0.001f, bottom * 1.0e-8f);
    if (gn > start + eps)
      gd = gn;
    else if (gf > start + eps)
      gd = gf;
    if (gd < end) {
      end = gd;
      ground = true;
    }
  }
}
__device__ __forceinline__ void aerial_prefix(const DevParams& P, float h, float cosv, float bottom, float& start,
                                              float& end, bool& valid) {
  bool v, g;
  segment_from_altitude(P, h, cosv, bottom, start, end, v, g);
  if (v && !g) {
    float closest = -(bottom + h) * cosv;
    if (closest > start && closest < end) end = closest;
  }
  valid = v && end > start;
}

// ---- per-ray geometry ---------------------------------------------------------
// a + b = s + err exactly (Knuth's two-sum; no contraction applies to it).
__device__ __forceinline__ float two_sum(float a, float b, float& err) {
  const float s = a + b;
  const float bb = s - a;
  err = (a - (s - bb)) + (b - bb);
  return s;
}
// r(t)^2 - R^2 along a camera ray, t the distance from the camera at
// (0, R + h0, 0), is the quadratic q(u) = (q0 + q1 u) + u^2, u = t - t0.
// Cameras within half a planet radius of the ground use the reference's own
// coefficients about the camera (t0 = 0: _altitude_on_ray :237-262,
// _shell_roots_from_altitude :264-301).  Farther out, every sample is far
// from the camera and those terms, ~r_cam^2, cancel down to r^2 - R^2 ~ R H:
// float keeps no digit of a grazing ray's altitude (a 50 km planet seen from
// 1800 km: 10 m altitude errors against a 300 m Mie scale height, the
// reference's own float result then off by tens of percent).  Such rays
// pivot at the closest approach t_c = -(R + h0) cos v, where q0 = r_c^2 - R^2
// and the shell discriminants are differences of squares formed once per ray
// from the ray's sine in compensated float (r_c = (R + h0) sin v as an
// unevaluated sum hi + lo: Knuth's two-sum and the FMA two-product), which
// keeps r_c^2 - R^2 and (R + top)^2 - r_c^2 to a few float ulps of themselves
// at every grazing angle without FP64 (a small fraction of the FP32 rate on
// this part).
struct RayGeom {
  float h0, cosv;    // camera altitude, view cosine
  float t0, q0, q1;  // pivot and coefficients of q
  float tc;          // closest-approach distance
  float disc_top, disc_ground;  // far: (shell radius)^2 - r_c^2 of the top and the ground
  bool far;          // pivot at t_c (far_camera)
};
// Camera far enough for the closest-approach pivot: above the shell and more
// than half a planet radius up.
__device__ __forceinline__ bool far_camera(const DevParams& P, float bottom, float h0) {
  return h0 > P.top && h0 > 0.5f * bottom;
}
__device__ __forceinline__ RayGeom ray_geom(const DevParams& P, float bottom, float h0, float cosv, float sinv) {
  RayGeom G;
  G.h0 = h0;
  G.cosv = cosv;
  const float a = mx(h0, 0.0f);
  G.far = far_camera(P, bottom, a);
  if (!G.far) {
    const float orad = bottom + a;
    G.t0 = 0.0f;
    G.q0 = a * (2.0f * bottom + a);
    G.q1 = 2.0f * orad * cosv;
    G.tc = -orad * cosv;
    G.disc_top = G.disc_ground = 0.0f;
  } else {
    float o_lo, bt_lo;
    const float o = two_sum(bottom, a, o_lo);         // R + h0 = o + o_lo
    const float rc = o * sinv;                         // r_c = rc + rc_lo
    const float rc_lo = fmaf(o, sinv, -rc) + o_lo * sinv;
    const float bt = two_sum(bottom, P.top, bt_lo);    // R + top = bt + bt_lo
    // R - r_c and (R + top) - r_c: the leading differences are exact where
    // they cancel (Sterbenz), the low parts then carry the digits
    const float dg = (bottom - rc) - rc_lo;
    const float dt = ((bt - rc) + bt_lo) - rc_lo;
    G.disc_ground = dg * (bottom + rc);
    G.disc_top = dt * (bt + rc);
    G.t0 = G.tc = -fmaf(o, cosv, o_lo * cosv);
    G.q0 = -G.disc_ground;
    G.q1 = 0.0f;
  }
  return G;
}
// Altitude at distance t along the ray (the reference's form of :237-262).
__device__ __forceinline__ float altitude_at(const RayGeom& G, float t, float bottom) {
  const float u = t - G.t0;
  const float delta = (G.q0 + G.q1 * u) + u * u;
  const float len = fsqrt(mx(bottom * bottom + delta, 0.0f));
  return fdiv(delta, mx(len + bottom, 1.0f));
}
// Cosine between the ray and the local vertical at distance t, r = R + h.
__device__ __forceinline__ float vertical_cosine_at(const RayGeom& G, float t, float radius) {
  return (t - G.tc) * frcp(mx(radius, 1.0f));
}
// Roots of the ray with the sphere of radius bottom + shell.
__device__ __forceinline__ void shell_roots_g(const RayGeom& G, float shell, float bottom, float& nearv, float& farv,
                                              bool& hit) {
  if (!G.far) {
    shell_roots(G.h0, G.cosv, shell, bottom, nearv, farv, hit);
    return;
  }
  const float disc = shell > 0.0f ? G.disc_top : G.disc_ground;  // shell is the top or 0
  hit = disc >= 0.0f;
  nearv = kLargeF;
  farv = -kLargeF;
  if (hit) {
    const float root = sqrtf(disc);
    nearv = G.tc - root;
    farv = G.tc + root;
  }
}
// _atmosphere_segment_from_altitude :303-340 on a ray's geometry.
__device__ __forceinline__ void segment_of(const DevParams& P, const RayGeom& G, float bottom, float& start,
                                           float& end, bool& valid, bool& ground) {
  if (!G.far) {
    segment_from_altitude(P, G.h0, G.cosv, bottom, start, end, valid, ground);
    return;
  }
  float on, of;
  bool oh;
  shell_roots_g(G, P.top, bottom, on, of, oh);
  start = mx(on, 0.0f);
  end = of;
  valid = oh && end > start;
  ground = false;
  float gn, gf;
  bool gh;
  shell_roots_g(G, 0.0f, bottom, gn, gf, gh);
  if (valid && gh) {
    float gd = kLargeF;
    if (gn > start + 1.0e-3f)
      gd = gn;
    else if (gf > start + 1.0e-3f)
      gd = gf;
    if (gd < end) {
      end = gd;
      ground = true;
    }
  }
}
// _aerial_prefix_segment_from_altitude :376-395 on a ray's geometry.
__device__ __forceinline__ void aerial_prefix_of(const DevParams& P, const RayGeom& G, float bottom, float& start,
                                                 float& end, bool& valid) {
  bool v, g;
  segment_of(P, G, bottom, start, end, v, g);
  if (v && !g && G.tc > start && G.tc < end) end = G.tc;
  valid = v && end > start;
}
__device__ __forceinline__ float distance_to_top(const DevParams& P, float h, float cosv, float bottom) {
  float radius = bottom + mx(h, 0.0f);
  float delta = (P.top - h) * ((2.0f * bottom + P.top) + h);
  float disc = radius * radius * cosv * cosv + delta;
  return mx(-radius * cosv + fsqrt(mx(disc, 0.0f)), 0.0f);
}

// ---- LUT parameterisations (:410-568) ---------------------------------------
__device__ __forceinline__ void t_uv_to_ray(const DevParams& P, float u, float v, float bottom, float& h,
                                            float& cosv, float& dist) {
  float sh = shell_rho(P.top, bottom);
  float rho = sh * clampf(v, 0.0f, 1.0f);
  float rl = sqrtf(rho * rho + bottom * bottom);
  h = rho * rho / mx(rl + bottom, 1.0f);
  float radius = bottom + h;
  float dmin = P.top - h;
  float dmax = rho + sh;
  dist = dmin + clampf(u, 0.0f, 1.0f) * (dmax - dmin);
  float c = 1.0f;
  if (dist > 1.0e-6f) c = ((P.top - h) * ((2.0f * bottom + P.top) + h) - dist * dist) / (2.0f * radius * dist);
  cosv = clampf(c, -1.0f, 1.0f);
}
__device__ __forceinline__ void t_ray_to_uv(const DevParams& P, float h, float cosv, float bottom, float sh,
                                            float inv_sh, float& u, float& v, float rho_known = -1.0f) {
  // rho_known: shell_rho(h) already evaluated by the caller for h in [0, top]
  const bool inside = h >= 0.0f && h <= P.top;
  h = clampf(h, 0.0f, P.top);
  float rho = (inside && rho_known >= 0.0f) ? rho_known : shell_rho(h, bottom);
  float d = distance_to_top(P, h, cosv, bottom);
  float dmin = P.top - h;
  float dmax = rho + sh;
  u = __saturatef(fdiv(d - dmin, mx(dmax - dmin, 1.0e-6f)));
  v = __saturatef(rho * inv_sh);
}
__device__ __forceinline__ float warp_boundary(float closest_raw, float start, float end, float f) {
  float closest = clampf(closest_raw, start, end);
  float eps = mx((end - start) * 1.0e-6f, 1.0e-5f);
  if (closest <= start + eps) return start + (end - start) * f * f;
  if (closest >= end - eps) {
    float inv = 1.0f - f;
    return end - (end - start) * inv * inv;
  }
  if (f < 0.5f) {
    float inv = 1.0f - f * 2.0f;
    return closest - (closest - start) * inv * inv;
  }
  float local = f * 2.0f - 1.0f;
  return closest + (end - closest) * local * local;
}
// Warped interval boundaries of one ray: the branch of warp_boundary depends
// only on the ray's closest-approach distance and interval, so it is taken
// once per ray; each boundary then costs the reference's own expression.
struct RayWarp {
  int mode;  // 0: dense at start, 1: dense at end, 2: dense around the closest point
  float start, end, closest;
};
__device__ __forceinline__ RayWarp make_warp(float closest_raw, float start, float end) {
  RayWarp w;
  w.start = start;
  w.end = end;
  w.closest = clampf(closest_raw, start, end);
  float eps = mx((end - start) * 1.0e-6f, 1.0e-5f);
  w.mode = w.closest <= start + eps ? 0 : (w.closest >= end - eps ? 1 : 2);
  return w;
}
__device__ __forceinline__ float warp_at(const RayWarp& w, float f) {
  if (w.mode == 0) return w.start + (w.end - w.start) * f * f;
  if (w.mode == 1) {
    float inv = 1.0f - f;
    return w.end - (w.end - w.start) * inv * inv;
  }
  if (f < 0.5f) {
    float inv = 1.0f - f * 2.0f;
    return w.closest - (w.closest - w.start) * inv * inv;
  }
  float local = f * 2.0f - 1.0f;
  return w.closest + (w.end - w.closest) * local * local;
}

__device__ __forceinline__ float horizon_cosine(float h, float bottom) {
  float radius = bottom + mx(h, 0.0f);
  return fdiv(-shell_rho(h, bottom), mx(radius, 1.0f));
}
__device__ __forceinline__ float sky_horizon_zenith(float h, float bottom) {
  float a = mx(h, 0.0f);
  float radius = bottom + a;
  float tc = shell_rho(a, bottom) / mx(radius, 1.0f);
  return kPiF - acosf(clampf(tc, 0.0f, 1.0f));
}
__device__ __forceinline__ float sky_v_to_zenith(float v, float hz) {
  if (v < 0.5f) {
    float inv = 1.0f - 2.0f * v;
    return hz * (1.0f - inv * inv);
  }
  float local = 2.0f * v - 1.0f;
  return hz + (kPiF - hz) * local * local;
}
__device__ __forceinline__ float sky_zenith_to_v(float z, float hz) {
  if (z < hz) {
    float n = clampf(z / mx(hz, 1.0e-6f), 0.0f, 1.0f);
    return 0.5f * (1.0f - sqrtf(mx(1.0f - n, 0.0f)));
  }
  float n = clampf((z - hz) / mx(kPiF - hz, 1.0e-6f), 0.0f, 1.0f);
  return 0.5f + 0.5f * sqrtf(n);
}
__device__ __forceinline__ float sun_u_to_cosine(float u, float h, float bottom) {
  float hc = horizon_cosine(h, bottom);
  float c;
  if (u < 0.5f) {
    float inv = 1.0f - 2.0f * u;
    c = hc - (hc + 1.0f) * inv * inv;
  } else {
    float local = 2.0f * u - 1.0f;
    c = hc + (1.0f - hc) * local * local;
  }
  return clampf(c, -1.0f, 1.0f);
}
__device__ __forceinline__ float sun_cosine_to_u(float c, float hc) {
  if (c < hc) {
    float n = __saturatef(fdiv(hc - c, mx(hc + 1.0f, 1.0e-6f)));
    return 0.5f * (1.0f - fsqrt(n));
  }
  float n = __saturatef(fdiv(c - hc, mx(1.0f - hc, 1.0e-6f)));
  return 0.5f + 0.5f * fsqrt(n);
}

// ---- LUT sampling -----------------------------------------------------------
// Bilinear tap with the reference's half-texel rule and edge clamp
// (:618-640, :655-683, :1503-1525).
__device__ __forceinline__ f3 bilinear(const float4* __restrict__ lut, int w, int h, float u, float v) {
  float x = clampf(u * float(w) - 0.5f, 0.0f, float(w - 1));
  float y = clampf(v * float(h) - 0.5f, 0.0f, float(h - 1));
  const float xf = floorf(x), yf = floorf(y);
  int x0 = int(xf);
  int y0 = int(yf);
  int x1 = min(x0 + 1, w - 1);
  int y1 = min(y0 + 1, h - 1);
  float fx = x - xf;
  float fy = y - yf;
  f3 a = from4(__ldg(lut + y0 * w + x0));
  f3 b = from4(__ldg(lut + y0 * w + x1));
  f3 c = from4(__ldg(lut + y1 * w + x0));
  f3 d = from4(__ldg(lut + y1 * w + x1));
  f3 lo = a * (1.0f - fx) + b * fx;
  f3 hi = c * (1.0f - fx) + d * fx;
  return lo * (1.0f - fy) + hi * fy;
}

// Per-launch geometry shared by every sample of a kernel.
struct Frame {
  const float4* __restrict__ tlut;
  const float4* __restrict__ mslut;
  float bottom;     // planet radius (f32)
  float shell_top;  // shell_rho(top, bottom)
  float ar;         // sun angular radius (rad)
  f3 sun;
  f3 E;             // solar irradiance
  float inv_shell_top;
  float cos_ar, sin_ar;  // of the sun's angular radius
};
__device__ __forceinline__ Frame make_frame(const DevParams& P, const float4* tlut, const float4* mslut,
                                            float bottom, float ar, f3 sun, f3 E) {
  Frame F;
  F.tlut = tlut;
  F.mslut = mslut;
  F.bottom = bottom;
  F.shell_top = sqrtf(mx(P.top, 0.0f) * (2.0f * bottom + mx(P.top, 0.0f)));
  F.ar = ar;
  F.sun = sun;
  F.E = E;
  F.inv_shell_top = 1.0f / mx(F.shell_top, 1.0e-6f);
  // thresholds of the whole-disk tests only: intrinsic accuracy suffices
  F.sin_ar = __sinf(ar);
  F.cos_ar = __cosf(ar);
  return F;
}

// _sample_transmittance_unoccluded :609-640
__device__ __forceinline__ f3 sample_t(const DevParams& P, const Frame& F, float h, float cosv,
                                       float rho_known = -1.0f) {
  float u, v;
  t_ray_to_uv(P, mx(h, 0.0f), cosv, F.bottom, F.shell_top, F.inv_shell_top, u, v, rho_known);
  return bilinear(F.tlut, P.t_w, P.t_h, u, v);
}
// _sample_multi_scattering :642-683
__device__ __forceinline__ f3 sample_ms(const DevParams& P, const Frame& F, float h, float sc, float hc) {
  float af = __saturatef(h * P.inv_top);
  float u = sun_cosine_to_u(sc, hc);
  float v = fsqrt(af);
  return bilinear(F.mslut, P.ms_w, P.ms_h, u, v);
}

// Horizon at one sample altitude: cosine hc = -rho/r of the horizon
// zenith, and sin of that zenith, R/r (rho^2 = r^2 - R^2).
struct Horizon {
  float hc;        // horizon cosine
  float sin_hz;    // sine of the horizon zenith
  float rho;       // shell_rho(h)
};
__device__ __forceinline__ Horizon horizon_at(float h, float bottom) {
  Horizon H;
  float radius = bottom + mx(h, 0.0f);
  float inv_r = frcp(mx(radius, 1.0f));
  H.rho = shell_rho(h, bottom);
  H.hc = -H.rho * inv_r;
  H.sin_hz = mn(bottom * inv_r, 1.0f);
  return H;
}
// _solar_disk_visibility :728-754, given horizon and sun zenith angles
__device__ __forceinline__ float disk_visibility(float hz, float sz, float ar) {
  float n = clampf(fdiv(hz - sz, mx(ar, 1.0e-6f)), -1.0f, 1.0f);
  return (acosf(-n) + n * sqrtf(mx(1.0f - n * n, 0.0f))) * (1.0f / kPiF);
}
// _sample_solar_transmittance :756-789 (returns the disk visibility too).
// The reference compares the horizon and sun zenith angles; whole-disk
// cases are decided here in cosine space without acos:
//   disk fully above the horizon  <=> sz <= hz - ar <=> cos sz >= cos(hz - ar)
//   disk fully below the horizon  <=> sz >= hz + ar <=> cos sz <= cos(hz + ar)
// with cos(hz -+ ar) = hc cos ar +- sin hz sin ar.  There the reference's
// visibility is exactly 1 (its representative zenith is then the sun's own,
// whose cosine is sc) or exactly 0; within float rounding of the thresholds
// its visibility differs from 1 or 0 by < 1e-6.  Only the penumbra band
// evaluates the reference's acos formulation.
__device__ __forceinline__ f3 sample_solar_t(const DevParams& P, const Frame& F, float h, float sc, Horizon H,
                                             float& vis) {
  const float cs = clampf(sc, -1.0f, 1.0f);
  const float a = H.hc * F.cos_ar;
  const float b = H.sin_hz * F.sin_ar;
  if (cs >= a + b) {
    vis = 1.0f;
    return sample_t(P, F, h, cs, H.rho);
  }
  if (cs <= a - b && H.hc >= -F.cos_ar) {  // hz + ar <= pi
    vis = 0.0f;
    return splat(0.0f);
  }
  const float hz = acosf(clampf(H.hc, -1.0f, 1.0f));
  const float sz = acosf(cs);
  vis = disk_visibility(hz, sz, F.ar);
  const float rz = mn(sz, hz - F.ar * 0.25f);
  const float rc = cosf(mx(rz, 0.0f));
  return sample_t(P, F, h, rc, H.rho) * vis;
}
// _rayleigh_phase / _mie_phase :791-804
__device__ __forceinline__ float rayleigh_phase(const DevParams& P, float c) {
  return 3.0f * (1.0f + c * c) / P.ray_k;
}
__device__ __forceinline__ float mie_phase(const DevParams& P, float c) {
  float den = mx(P.mie_c1 - P.mie_c2 * c, 1.0e-8f);
  return P.mie_k1 * (1.0f + c * c) / (P.mie_k2 * (den * sqrtf(den)));
}
// In-scattering weight (1 - T) / ext of one segment, T = exp(-x), x =
// ext * step.  The reference forms 1 - T directly, which cancels in f32 when
// x is small: centimetre segments next to a camera standing on the ground
// give x ~ 1e-7 and a weight with no significant digit left (its own f32
// result is then percents away from its f64 one).  Below x = 1/32 the weight
// is the Taylor series step * (1 - x/2 + x^2/6 - x^3/24) of the same quantity
// (truncation under 1e-8 relative; step itself at ext = 0, as the
// reference's ext <= 1e-12 branch); above it 1 - T keeps 5+ digits.
__device__ __forceinline__ float in_scatter_weight(float ext, float step, float x, float tr) {
  if (x < 0.03125f) return step * fmaf(x, fmaf(x, fmaf(x, -1.0f / 24.0f, 1.0f / 6.0f), -0.5f), 1.0f);
  return fdiv(1.0f - tr, ext);
}
// _segment_integral :806-816
__device__ __forceinline__ void segment_integral(f3 ext, float step, f3& tr, f3& integ) {
  // __expf: ~2 ulp near 0 (as expf), up to ~95 ulp at the clamp (T ~ 1e-35)
  const f3 x = vmin(ext * step, 80.0f);
  tr = {__expf(-x.x), __expf(-x.y), __expf(-x.z)};
  integ.x = in_scatter_weight(ext.x, step, x.x, tr.x);
  integ.y = in_scatter_weight(ext.y, step, x.y, tr.y);
  integ.z = in_scatter_weight(ext.z, step, x.z, tr.z);
}

// Per-ray constants of the constant-source samples (everything of
// _scattering_source :818-856 that does not depend on the sample).
struct RaySource {
  float t0, q0, q1;  // the ray's altitude quadratic (RayGeom)
  float s0;          // (origin + t0 ray) . sun
  float r_sun;       // ray . sun
  f3 ER, EM;         // E * beta_R * phase_R, E * beta_Ms * phase_M
};
__device__ __forceinline__ RaySource make_ray_source(const DevParams& P, const Frame& F, const RayGeom& G, f3 ray) {
  RaySource R;
  R.t0 = G.t0;
  R.q0 = G.q0;
  R.q1 = G.q1;
  R.r_sun = dot(ray, F.sun);
  const float o_y = F.bottom + mx(G.h0, 0.0f);
  if (G.far) {
    // p(t0) . sun with the closest-approach point formed first (one rounding
    // per component, each ~r_c): o_y sun.y + t0 ray . sun cancels ~r_cam
    // down to ~r_c
    const f3 c = mk(G.t0 * ray.x, fmaf(G.t0, ray.y, o_y), G.t0 * ray.z);
    R.s0 = dot(c, F.sun);
  } else {
    R.s0 = o_y * F.sun.y;
  }
  const float cr = clampf(R.r_sun, -1.0f, 1.0f);
  R.ER = F.E * arr3(P.beta_r) * rayleigh_phase(P, cr);
  R.EM = F.E * arr3(P.beta_ms) * mie_phase(P, cr);
  return R;
}

// One constant-source segment [start, end] of the ray: _scattering_segment
// :858-899 with _scattering_source :818-856.  Returns (L, T) and the finite
// disk visibility at the sample.  The sample's radius is bottom + h (its
// altitude on the ray) and its sun cosine (p(t0) . sun + (t - t0) ray . sun) /
// radius; the reference forms the point first - same quantities, rounding
// differs in the last bits.
template <bool kMultiple>
__device__ __forceinline__ Seg source_segment(const DevParams& P, const Frame& F, const RaySource& R, float start,
                                              float end, float& vis) {
  float step = mx(end - start, 0.0f);
  float dist = (start + end) * 0.5f;
  const float u = dist - R.t0;
  const float delta = (R.q0 + R.q1 * u) + u * u;
  float h = fdiv(delta, mx(fsqrt(mx(F.bottom * F.bottom + delta, 0.0f)) + F.bottom, 1.0f));
  Density d = density(P, h);
  f3 ext = extinction_of(P, d);
  Seg s;
  f3 integ;
  segment_integral(ext, step, s.T, integ);
  const float radius = F.bottom + h;
  const float sc = (R.s0 + u * R.r_sun) * frcp(mx(radius, 1.0f));
  Horizon H = horizon_at(h, F.bottom);
  f3 st = sample_solar_t(P, F, h, sc, H, vis);
  f3 src = st * (R.ER * d.r + R.EM * d.m);
  if (kMultiple) src = src + scattering_of(P, d) * sample_ms(P, F, h, sc, H.hc);
  s.L = src * integ;
  return s;
}

}  // namespace atm
