// atm_oracle.cpp - CPU restatement of the reference atmosphere path.
//
// TEST INFRASTRUCTURE ONLY.  This is the parity oracle for the CUDA kernels:
// tests, the smoke check and the bench's CPU-baseline leg load it; the
// product never does.  It restates, function for function, the Taichi code of
// src/planet_renderer/atmosphere/renderer.py (reference file; line numbers
// below refer to it) in plain scalar C++, templated on the scalar type:
//   Real = float   mirrors Taichi with default_fp = f32: every Python float
//                  constant is rounded to float where it meets an f32 value,
//                  constant-only sub-expressions are folded in double (the
//                  Taichi trace evaluates them in Python), no FMA
//                  contraction (built with -ffp-contract=off);
//   Real = double  the same algorithm and the same step counts in FP64.
// Pinned against golden vectors produced by running the reference's own
// kernel source (tests/golden/make_golden.py).
//
// Build: oracle/build_oracle.py (g++ -O3 -fopenmp -ffp-contract=off).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "atm_capi.h"

#ifdef _OPENMP
#include <omp.h>
#endif

// 1: the segment weight by its Taylor series where it cancels (not the
// reference; see Model::series_weight).
static int g_series_weight = 0;

// Scalar arguments of the composite kernel (reference _composite :1827-1849);
// values as the host passes them (Python floats), rounded on use.
struct CompositeArgs {
  int32_t width, height, diagnostic_view;
  double bottom, cam_alt, sky_alt, ar, tanfov, star_start, star_end;
  double sun[3], E[3], disk[3], right[3], up[3], fwd[3];
};

namespace {

constexpr double kPi = 3.141592653589793;     // math.pi (renderer.py:12)
constexpr double kLarge = 1.0e30;             // _LARGE_DISTANCE (:13)


// Math entry points: plain libm for float/double, overloads for the counting
// type below (found by argument-dependent lookup).
template <class R> inline R m_sqrt(R x) { using std::sqrt; return sqrt(x); }
template <class R> inline R m_exp(R x) { using std::exp; return exp(x); }
template <class R> inline R m_acos(R x) { using std::acos; return acos(x); }
template <class R> inline R m_cos(R x) { using std::cos; return cos(x); }
template <class R> inline R m_sin(R x) { using std::sin; return sin(x); }
template <class R> inline R m_pow(R x, R y) { using std::pow; return pow(x, y); }
template <class R> inline R m_atan2(R y, R x) { using std::atan2; return atan2(y, x); }
template <class R> inline R m_fabs(R x) { using std::fabs; return fabs(x); }
template <class R> inline R m_floor(R x) { using std::floor; return floor(x); }
template <class R> inline double as_d(R x) { return double(x); }
// Smallest distance (m) of any density evaluation's altitude from the
// profile's cutoffs (0 and the shell top, where _density drops to zero) since
// the calling thread last reset it: the composite reports it per pixel.  A
// radiance sample that close to a cutoff switches its density on or off
// under a rounding of its altitude, so two float evaluations of the same
// pixel can differ there by that sample's whole contribution.
thread_local double g_cutoff_margin = HUGE_VAL;

template <class R>
struct V3 {
  R x, y, z;
};
template <class R> inline V3<R> v3(R x, R y, R z) { return {x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline V3<R> operator/(V3<R> a, V3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class R> inline R norm(V3<R> a) { return m_sqrt(dot(a, a)); }
template <class R> inline R mx(R a, R b) { return a > b ? a : b; }  // ti.max
template <class R> inline R mn(R a, R b) { return a < b ? a : b; }  // ti.min
template <class R> inline R clampr(R x, R lo, R hi) { return mn(mx(x, lo), hi); }
template <class R> inline V3<R> vmax(V3<R> a, R s) { return {mx(a.x, s), mx(a.y, s), mx(a.z, s)}; }
template <class R> inline V3<R> vmin(V3<R> a, R s) { return {mn(a.x, s), mn(a.y, s), mn(a.z, s)}; }
template <class R> inline V3<R> vclamp(V3<R> a, R lo, R hi) { return vmin(vmax(a, lo), hi); }
template <class R> inline V3<R> vexp(V3<R> a) { return {m_exp(a.x), m_exp(a.y), m_exp(a.z)}; }
template <class R> inline V3<R> splat(R s) { return {s, s, s}; }

// Read-only LUT views in the Taichi field layout (W, H[, D], 3).
template <class R>
struct Lut2 {
  const R* data;
  int w, h;
  V3<R> at(int x, int y) const {
    const R* p = data + (static_cast<size_t>(x) * h + y) * 3;
    return {p[0], p[1], p[2]};
  }
};
template <class R>
struct Lut3 {
  const R* data;
  int w, h, d;
  V3<R> at(int x, int y, int z) const {
    const R* p = data + ((static_cast<size_t>(x) * h + y) * d + z) * 3;
    return {p[0], p[1], p[2]};
  }
};

template <class R>
struct Model {
  const AtmParams& P;
  Lut2<R> tlut{nullptr, 0, 0};
  Lut2<R> mslut{nullptr, 0, 0};
  Lut2<R> svlut{nullptr, 0, 0};
  Lut3<R> aplut{nullptr, 0, 0, 0};
  explicit Model(const AtmParams& p) : P(p) {}

  R top() const { return R(P.top_altitude_m); }
  V3<R> beta_r() const { return v3(R(P.rayleigh_scattering_per_m[0]), R(P.rayleigh_scattering_per_m[1]), R(P.rayleigh_scattering_per_m[2])); }
  V3<R> beta_ms() const { return v3(R(P.mie_scattering_per_m[0]), R(P.mie_scattering_per_m[1]), R(P.mie_scattering_per_m[2])); }
  V3<R> beta_me() const { return v3(R(P.mie_extinction_per_m[0]), R(P.mie_extinction_per_m[1]), R(P.mie_extinction_per_m[2])); }
  V3<R> beta_o() const { return v3(R(P.absorption_extinction_per_m[0]), R(P.absorption_extinction_per_m[1]), R(P.absorption_extinction_per_m[2])); }
  V3<R> albedo() const { return v3(R(P.ground_albedo[0]), R(P.ground_albedo[1]), R(P.ground_albedo[2])); }

  // _density :168-192
  V3<R> density(R h) const {
    const double hd = as_d(h);
    g_cutoff_margin = std::min(g_cutoff_margin, std::min(std::fabs(hd), std::fabs(hd - P.top_altitude_m)));
    R ray = R(0), mie = R(0), ozone = R(0);
    if (R(0) <= h && h <= top()) {
      ray = m_exp(-h / R(P.rayleigh_scale_height_m));
      mie = m_exp(-h / R(P.mie_scale_height_m));
      ozone = mx(R(1) - m_fabs(h - R(P.absorption_peak_altitude_m)) / R(P.absorption_half_width_m), R(0));
    }
    return {ray, mie, ozone};
  }
  // _extinction :194-201
  V3<R> extinction(R h) const {
    V3<R> d = density(h);
    return (beta_r() * d.x + beta_me() * d.y) + beta_o() * d.z;
  }
  // _scattering :203-209
  V3<R> scattering(R h) const {
    V3<R> d = density(h);
    return beta_r() * d.x + beta_ms() * d.y;
  }
  // _sphere_roots :211-226
  void sphere_roots(V3<R> o, V3<R> d, R radius, R& nearv, R& farv, bool& hit) const {
    R projected = dot(o, d);
    R perpendicular = norm(o - d * projected);
    R clearance = radius - perpendicular;
    hit = clearance >= R(0);
    nearv = R(kLarge);
    farv = -R(kLarge);
    if (hit) {
      R disc = mx(clearance, R(0)) * (radius + perpendicular);
      R root = m_sqrt(mx(disc, R(0)));
      nearv = -projected - root;
      farv = -projected + root;
    }
  }
  // _shell_rho :228-235
  R shell_rho(R h, R bottom) const {
    R a = mx(h, R(0));
    return m_sqrt(a * (R(2) * bottom + a));
  }
  // _altitude_on_ray :237-262
  R altitude_on_ray(R h0, R cosv, R t, R bottom) const {
    R a = mx(h0, R(0));
    R orad = bottom + a;
    R delta = (a * (R(2) * bottom + a) + R(2) * orad * cosv * t) + t * t;
    R len = m_sqrt(mx(bottom * bottom + delta, R(0)));
    return delta / mx(len + bottom, R(1));
  }
  // _shell_roots_from_altitude :264-301
  void shell_roots(R h0, R cosv, R shell, R bottom, R& nearv, R& farv, bool& hit) const {
    R orad = bottom + h0;
    R hl = orad * cosv;
    R c = (h0 - shell) * ((R(2) * bottom + h0) + shell);
    R disc = hl * hl - c;
    hit = disc >= R(0);
    nearv = R(kLarge);
    farv = -R(kLarge);
    if (hit) {
      R root = m_sqrt(mx(disc, R(0)));
      R sign = hl < R(0) ? R(-1) : R(1);
      R q = -hl - sign * root;
      R r0 = -hl - root;
      R r1 = -hl + root;
      if (m_fabs(q) > R(1.0e-12)) {
        r0 = q;
        r1 = c / q;
      }
      nearv = mn(r0, r1);
      farv = mx(r0, r1);
    }
  }
  // _atmosphere_segment_from_altitude :303-340
  void segment_from_altitude(R h, R cosv, R bottom, R& start, R& end, bool& valid, bool& ground) const {
    R on, of; bool oh;
    shell_roots(h, cosv, top(), bottom, on, of, oh);
    start = mx(on, R(0));
    end = of;
    valid = oh && end > start;
    ground = false;
    R gn, gf; bool gh;
    shell_roots(h, cosv, R(0), bottom, gn, gf, gh);
    if (valid && gh) {
      R gd = R(kLarge);
      const R eps = R(1.0e-3);
      if (gn > start + eps) gd = gn;
      else if (gf > start + eps) gd = gf;
      if (gd < end) { end = gd; ground = true; }
    }
  }
  // _atmosphere_segment :342-374
  void segment_vec(V3<R> o, V3<R> d, R bottom, R& start, R& end, bool& valid, bool& ground) const {
    R top_radius = bottom + top();
    R on, of; bool oh;
    sphere_roots(o, d, top_radius, on, of, oh);
    start = mx(on, R(0));
    end = of;
    valid = oh && end > start;
    ground = false;
    R gn, gf; bool gh;
    sphere_roots(o, d, bottom, gn, gf, gh);
    if (valid && gh) {
      R gd = R(kLarge);
      R eps = mx(R(0.001), bottom * R(1.0e-8));
      if (gn > start + eps) gd = gn;
      else if (gf > start + eps) gd = gf;
      if (gd < end) { end = gd; ground = true; }
    }
  }
  // _aerial_prefix_segment_from_altitude :376-395
  void aerial_prefix(R h, R cosv, R bottom, R& start, R& end, bool& valid) const {
    bool v, g;
    segment_from_altitude(h, cosv, bottom, start, end, v, g);
    if (v && !g) {
      R closest = -(bottom + h) * cosv;
      if (closest > start && closest < end) end = closest;
    }
    valid = v && end > start;
  }
  // _distance_to_top_atmosphere :397-408
  R distance_to_top(R h, R cosv, R bottom) const {
    R radius = bottom + mx(h, R(0));
    R delta = (top() - h) * ((R(2) * bottom + top()) + h);
    R disc = radius * radius * cosv * cosv + delta;
    return mx(-radius * cosv + m_sqrt(mx(disc, R(0))), R(0));
  }
  // _transmittance_uv_to_ray :410-432
  void t_uv_to_ray(R u, R v, R bottom, R& h, R& cosv, R& dist) const {
    R sh = shell_rho(top(), bottom);
    R rho = sh * clampr(v, R(0), R(1));
    R rl = m_sqrt(rho * rho + bottom * bottom);
    h = rho * rho / mx(rl + bottom, R(1));
    R radius = bottom + h;
    R dmin = top() - h;
    R dmax = rho + sh;
    dist = dmin + clampr(u, R(0), R(1)) * (dmax - dmin);
    R c = R(1);
    if (dist > R(1.0e-6))
      c = ((top() - h) * ((R(2) * bottom + top()) + h) - dist * dist) / (R(2) * radius * dist);
    cosv = clampr(c, R(-1), R(1));
  }
  // _transmittance_ray_to_uv :434-452
  void t_ray_to_uv(R h, R cosv, R bottom, R& u, R& v) const {
    h = clampr(h, R(0), top());
    R sh = shell_rho(top(), bottom);
    R rho = shell_rho(h, bottom);
    R d = distance_to_top(h, cosv, bottom);
    R dmin = top() - h;
    R dmax = rho + sh;
    u = (d - dmin) / mx(dmax - dmin, R(1.0e-6));
    v = rho / mx(sh, R(1.0e-6));
    u = clampr(u, R(0), R(1));
    v = clampr(v, R(0), R(1));
  }
  // _warped_interval_boundary :454-480
  R warp(V3<R> o, V3<R> d, R start, R end, R f) const {
    R closest = clampr(-dot(o, d), start, end);
    R dist = start;
    R eps = mx((end - start) * R(1.0e-6), R(1.0e-5));
    if (closest <= start + eps) {
      dist = start + (end - start) * f * f;
    } else if (closest >= end - eps) {
      R inv = R(1) - f;
      dist = end - (end - start) * inv * inv;
    } else if (f < R(0.5)) {
      R local = f * R(2);
      R inv = R(1) - local;
      dist = closest - (closest - start) * inv * inv;
    } else {
      R local = f * R(2) - R(1);
      dist = closest + (end - closest) * local * local;
    }
    return dist;
  }
  // _sky_horizon_zenith :482-490
  R sky_horizon_zenith(R h, R bottom) const {
    R a = mx(h, R(0));
    R radius = bottom + a;
    R tc = shell_rho(a, bottom) / mx(radius, R(1));
    return R(kPi) - m_acos(clampr(tc, R(0), R(1)));
  }
  // _sky_v_to_zenith :492-504
  R sky_v_to_zenith(R v, R h, R bottom) const {
    R hz = sky_horizon_zenith(h, bottom);
    if (v < R(0.5)) {
      R inv = R(1) - R(2) * v;
      return hz * (R(1) - inv * inv);
    }
    R local = R(2) * v - R(1);
    return hz + (R(kPi) - hz) * local * local;
  }
  // _sky_zenith_to_v :506-520
  R sky_zenith_to_v(R z, R h, R bottom) const {
    R hz = sky_horizon_zenith(h, bottom);
    if (z < hz) {
      R n = clampr(z / mx(hz, R(1.0e-6)), R(0), R(1));
      return R(0.5) * (R(1) - m_sqrt(mx(R(1) - n, R(0))));
    }
    R n = clampr((z - hz) / mx(R(kPi) - hz, R(1.0e-6)), R(0), R(1));
    return R(0.5) + R(0.5) * m_sqrt(n);
  }
  R horizon_cosine(R h, R bottom) const {
    R radius = bottom + mx(h, R(0));
    return -shell_rho(h, bottom) / mx(radius, R(1));
  }
  // _sun_u_to_cosine :522-542
  R sun_u_to_cosine(R u, R h, R bottom) const {
    R hc = horizon_cosine(h, bottom);
    R c = hc;
    if (u < R(0.5)) {
      R inv = R(1) - R(2) * u;
      c = hc - (hc + R(1)) * inv * inv;
    } else {
      R local = R(2) * u - R(1);
      c = hc + (R(1) - hc) * local * local;
    }
    return clampr(c, R(-1), R(1));
  }
  // _sun_cosine_to_u :544-568
  R sun_cosine_to_u(R c, R h, R bottom) const {
    R hc = horizon_cosine(h, bottom);
    if (c < hc) {
      R n = clampr((hc - c) / mx(hc + R(1), R(1.0e-6)), R(0), R(1));
      return R(0.5) * (R(1) - m_sqrt(n));
    }
    R n = clampr((c - hc) / mx(R(1) - hc, R(1.0e-6)), R(0), R(1));
    return R(0.5) + R(0.5) * m_sqrt(n);
  }
  // _integrate_extinction :570-607
  V3<R> integrate_extinction(V3<R> o, V3<R> d, R start, R end, R bottom) const {
    V3<R> od = splat(R(0));
    const int n = P.transmittance_steps;
    for (int i = 0; i < n; ++i) {
      R f0 = R(i) / R(n);
      R f1 = R(i + 1) / R(n);
      R d0 = warp(o, d, start, end, f0);
      R d1 = warp(o, d, start, end, f1);
      R step = d1 - d0;
      R dist = (d0 + d1) * R(0.5);
      R h = norm(o + d * dist) - bottom;
      od = od + extinction(h) * step;
    }
    return vexp(-vmin(od, R(80)));
  }
  // bilinear LUT sample with the half-texel rule (:618-640, :655-683, :1503-1525)
  static V3<R> bilinear(const Lut2<R>& L, R u, R v) {
    R x = clampr(u * R(L.w) - R(0.5), R(0), R(L.w - 1));
    R y = clampr(v * R(L.h) - R(0.5), R(0), R(L.h - 1));
    int x0 = static_cast<int>(m_floor(x));
    int y0 = static_cast<int>(m_floor(y));
    int x1 = std::min(x0 + 1, L.w - 1);
    int y1 = std::min(y0 + 1, L.h - 1);
    R fx = x - R(x0);
    R fy = y - R(y0);
    V3<R> lo = L.at(x0, y0) * (R(1) - fx) + L.at(x1, y0) * fx;
    V3<R> hi = L.at(x0, y1) * (R(1) - fx) + L.at(x1, y1) * fx;
    return lo * (R(1) - fy) + hi * fy;
  }
  // _sample_transmittance_unoccluded :609-640
  V3<R> sample_t(R h, R cosv, R bottom) const {
    R u, v;
    t_ray_to_uv(mx(h, R(0)), cosv, bottom, u, v);
    return bilinear(tlut, u, v);
  }
  // _sample_multi_scattering :642-683
  V3<R> sample_ms(R h, R sc, R bottom) const {
    R af = clampr(h / top(), R(0), R(1));
    R u = sun_cosine_to_u(sc, mx(h, R(0)), bottom);
    R v = m_sqrt(af);
    return bilinear(mslut, u, v);
  }
  // _solar_shadow_roots :685-726
  void shadow_roots(V3<R> o, V3<R> d, V3<R> sun, R bottom, R& r0, R& r1, int& v0, int& v1) const {
    V3<R> op = o - sun * dot(o, sun);
    V3<R> rp = d - sun * dot(d, sun);
    R quad = dot(rp, rp);
    R hl = dot(op, rp);
    R pl = norm(op);
    R c = (pl - bottom) * (pl + bottom);
    r0 = R(0); r1 = R(0); v0 = 0; v1 = 0;
    R disc = hl * hl - quad * c;
    if (quad > R(1.0e-8) && disc >= R(0)) {
      R sr = m_sqrt(mx(disc, R(0)));
      r0 = (-hl - sr) / quad;
      r1 = (-hl + sr) / quad;
      V3<R> p0 = o + d * r0;
      V3<R> p1 = o + d * r1;
      if (dot(p0, sun) < R(0)) v0 = 1;
      if (dot(p1, sun) < R(0)) v1 = 1;
    }
  }
  // _solar_disk_visibility :728-754
  R disk_visibility(R h, R sc, R bottom, R ar) const {
    R hc = horizon_cosine(h, bottom);
    R hz = m_acos(clampr(hc, R(-1), R(1)));
    R sz = m_acos(clampr(sc, R(-1), R(1)));
    R sep = hz - sz;
    R n = clampr(sep / mx(ar, R(1.0e-6)), R(-1), R(1));
    return (m_acos(-n) + n * m_sqrt(mx(R(1) - n * n, R(0)))) / R(kPi);
  }
  // _sample_solar_transmittance :756-789
  V3<R> sample_solar_t(R h, R sc, R bottom, R ar) const {
    R vis = disk_visibility(h, sc, bottom, ar);
    R hc = horizon_cosine(h, bottom);
    R hz = m_acos(clampr(hc, R(-1), R(1)));
    R sz = m_acos(clampr(sc, R(-1), R(1)));
    R rz = mn(sz, hz - ar * R(0.25));
    R rc = m_cos(mx(rz, R(0)));
    return sample_t(h, rc, bottom) * vis;
  }
  // _rayleigh_phase :791-793
  R rayleigh_phase(R c) const { return R(3) * (R(1) + c * c) / R(16.0 * kPi); }
  // _mie_phase :795-804
  R mie_phase(R c) const {
    const double g = P.mie_phase_g;  // a Python float: constant terms fold in double
    R den = mx(R(1.0 + g * g) - R(2.0 * g) * c, R(1.0e-8));
    return R(3.0 * (1.0 - g * g)) * (R(1) + c * c) / (R(8.0 * kPi * (2.0 + g * g)) * m_pow(den, R(1.5)));
  }
  // _segment_integral :806-816
  void segment_integral(V3<R> ext, R step, V3<R>& tr, V3<R>& integ) const {
    tr = vexp(-vmin(ext * step, R(80)));
    integ.x = ext.x > R(1.0e-12) ? (R(1) - tr.x) / ext.x : step;
    integ.y = ext.y > R(1.0e-12) ? (R(1) - tr.y) / ext.y : step;
    integ.z = ext.z > R(1.0e-12) ? (R(1) - tr.z) / ext.z : step;
    if (g_series_weight) {
      integ.x = series_weight(ext.x, step, integ.x);
      integ.y = series_weight(ext.y, step, integ.y);
      integ.z = series_weight(ext.z, step, integ.z);
    }
  }
  // Not the reference: the weight (1 - exp(-x)) / ext by its Taylor series
  // below x = 1/32, where the reference's float formula cancels.  Enabled
  // only to show that this one step is what makes the reference's float
  // result drift from its double result next to the ground.
  R series_weight(R ext, R step, R plain) const {
    R x = mn(ext * step, R(80));
    if (!(x < R(0.03125))) return plain;
    return step * (R(1) + x * (R(-0.5) + x * (R(1.0 / 6.0) + x * R(-1.0 / 24.0))));
  }
  // _scattering_source :818-856
  V3<R> scattering_source(V3<R> point, R h, V3<R> ray, V3<R> sun, V3<R> E, R bottom, R ar, bool multiple) const {
    R radius = norm(point);
    V3<R> radial = point / mx(radius, R(1));
    V3<R> d = density(h);
    R sc = dot(radial, sun);
    V3<R> st = sample_solar_t(h, sc, bottom, ar);
    R scos = clampr(dot(ray, sun), R(-1), R(1));
    V3<R> src = (E * st) * (beta_r() * d.x * rayleigh_phase(scos) + beta_ms() * d.y * mie_phase(scos));
    if (multiple) src = src + scattering(h) * sample_ms(h, sc, bottom);
    return src;
  }
  // _scattering_segment :858-899
  void scattering_segment(V3<R> o, R h0, V3<R> ray, R start, R end, V3<R> sun, V3<R> E, R bottom, R ar,
                          V3<R>& L, V3<R>& T, int64_t* counter) const {
    R step = mx(end - start, R(0));
    R dist = (start + end) * R(0.5);
    V3<R> point = o + ray * dist;
    R orad = mx(norm(o), R(1));
    V3<R> oradial = o / orad;
    R h = altitude_on_ray(h0, dot(oradial, ray), dist, bottom);
    V3<R> ext = extinction(h);
    V3<R> integ;
    segment_integral(ext, step, T, integ);
    V3<R> src = scattering_source(point, h, ray, sun, E, bottom, ar, true);
    L = src * integ;
    if (counter) ++*counter;
  }
  // _terminator_refinement_weight :901-966
  R refinement_weight(V3<R> o, R h0, V3<R> ray, R start, R end, V3<R> sun, R bottom, R ar,
                      R sr0, R sr1, int sv0, int sv1) const {
    R mid = (start + end) * R(0.5);
    R iw = mx(end - start, R(1.0e-4));
    R cr = R(1.0e30);
    if (sv0 != 0) cr = mn(cr, m_fabs(mid - sr0));
    if (sv1 != 0) cr = mn(cr, m_fabs(mid - sr1));
    R prox = clampr(R(2) - cr / iw, R(0), R(1));
    prox = prox * prox * (R(3) - R(2) * prox);
    V3<R> point = o + ray * mid;
    R radius = mx(norm(point), R(1));
    V3<R> radial = point / radius;
    R orad = mx(norm(o), R(1));
    V3<R> oradial = o / orad;
    R h = altitude_on_ray(h0, dot(oradial, ray), mid, bottom);
    R vis = disk_visibility(h, dot(radial, sun), bottom, ar);
    R pen = R(4) * vis * (R(1) - vis);
    return mx(prox, pen);
  }
  // _integrate_adaptive_scattering_interval :968-1032
  void adaptive_interval(V3<R> o, R h0, V3<R> ray, R start, R end, V3<R> sun, V3<R> E, R bottom, R ar, R w,
                         V3<R>& L, V3<R>& T, int64_t* counter) const {
    V3<R> cL, cT;
    scattering_segment(o, h0, ray, start, end, sun, E, bottom, ar, cL, cT, counter);
    L = cL;
    T = cT;
    if (w > R(0)) {
      V3<R> fL = splat(R(0)), fT = splat(R(1));
      const int n = P.aerial_terminator_substeps;
      for (int k = 0; k < n; ++k) {
        R f0 = R(k) / R(n);
        R f1 = R(k + 1) / R(n);
        R cs = start + (end - start) * f0;
        R ce = start + (end - start) * f1;
        V3<R> chL, chT;
        scattering_segment(o, h0, ray, cs, ce, sun, E, bottom, ar, chL, chT, counter);
        fL = fL + fT * chL;
        fT = fT * chT;
      }
      L = cL * (R(1) - w) + fL * w;
      T = cT * (R(1) - w) + fT * w;
    }
  }
  // _sample_sky_view :1474-1525
  V3<R> sample_sky_view(V3<R> ray, V3<R> sun, R cam_alt, R bottom) const {
    R zen = m_acos(clampr(ray.y, R(-1), R(1)));
    R vl = m_sqrt(ray.x * ray.x + ray.z * ray.z);
    R sl = m_sqrt(sun.x * sun.x + sun.z * sun.z);
    R ra = R(0);
    if (vl > R(1.0e-6) && sl > R(1.0e-6))
      ra = m_acos(clampr((ray.x * sun.x + ray.z * sun.z) / (vl * sl), R(-1), R(1)));
    R u = ra / R(kPi);
    R v = sky_zenith_to_v(zen, cam_alt, bottom);
    return bilinear(svlut, u, v);
  }
  // _sample_aerial_field :1527-1571
  V3<R> sample_aerial_field(R su, R sv, R df) const {
    const Lut3<R>& F = aplut;
    R x = clampr(su * R(F.w) - R(0.5), R(0), R(F.w - 1));
    R y = clampr(sv * R(F.h) - R(0.5), R(0), R(F.h - 1));
    R z = clampr(df, R(0), R(1)) * R(F.d - 1);
    int x0 = static_cast<int>(m_floor(x)), y0 = static_cast<int>(m_floor(y)), z0 = static_cast<int>(m_floor(z));
    int x1 = std::min(x0 + 1, F.w - 1), y1 = std::min(y0 + 1, F.h - 1), z1 = std::min(z0 + 1, F.d - 1);
    R fx = x - R(x0), fy = y - R(y0), fz = z - R(z0);
    V3<R> a = F.at(x0, y0, z0) * (R(1) - fx) + F.at(x1, y0, z0) * fx;
    V3<R> b = F.at(x0, y1, z0) * (R(1) - fx) + F.at(x1, y1, z0) * fx;
    V3<R> c = F.at(x0, y0, z1) * (R(1) - fx) + F.at(x1, y0, z1) * fx;
    V3<R> e = F.at(x0, y1, z1) * (R(1) - fx) + F.at(x1, y1, z1) * fx;
    V3<R> lo = a * (R(1) - fy) + b * fy;
    V3<R> hi = c * (R(1) - fy) + e * fy;
    return lo * (R(1) - fz) + hi * fz;
  }
  // _sample_aerial_scattering :1573-1601
  V3<R> sample_aerial_scattering(R su, R sv, R dist, R cam_alt, V3<R> ray, R bottom) const {
    R s, e; bool valid;
    aerial_prefix(cam_alt, ray.y, bottom, s, e, valid);
    R df = R(0);
    if (valid) df = clampr((dist - s) / mx(e - s, R(1)), R(0), R(1));
    return sample_aerial_field(su, sv, df);
  }
  // _surface_segment_transmittance :1603-1665
  V3<R> surface_segment_t(V3<R> o, R h0, V3<R> ray, R sd, R bottom) const {
    V3<R> tr = splat(R(1));
    R on, of; bool oh;
    shell_roots(h0, ray.y, top(), bottom, on, of, oh);
    R s = mx(on, R(0));
    R e = mn(sd, of);
    if (oh && e > s) {
      V3<R> np = o + ray * s;
      V3<R> sp = o + ray * e;
      V3<R> rr = -ray;
      R nl = norm(np), sl = norm(sp);
      V3<R> nrad = np / mx(nl, R(1));
      V3<R> srad = sp / mx(sl, R(1));
      R na = altitude_on_ray(h0, ray.y, s, bottom);
      R sa = altitude_on_ray(h0, ray.y, e, bottom);
      V3<R> s2t = sample_t(sa, dot(srad, rr), bottom);
      V3<R> n2t = sample_t(na, dot(nrad, rr), bottom);
      tr = vclamp(s2t / vmax(n2t, R(1.0e-6)), R(0), R(1));
    }
    return tr;
  }
  // _integrate_surface_scattering :1667-1755
  V3<R> integrate_surface(V3<R> o, R h0, V3<R> ray, R sd, V3<R> sun, V3<R> E, R bottom, R ar, int64_t* counter) const {
    V3<R> rad = splat(R(0)), vT = splat(R(1));
    R on, of; bool oh;
    shell_roots(h0, ray.y, top(), bottom, on, of, oh);
    R s = mx(on, R(0));
    R e = mn(sd, of);
    if (oh && e > s) {
      R sr0, sr1; int sv0, sv1;
      shadow_roots(o, ray, sun, bottom, sr0, sr1, sv0, sv1);
      const int n = P.aerial_horizon_raymarch_steps;
      for (int i = 0; i < n; ++i) {
        R f0 = R(i) / R(n);
        R f1 = R(i + 1) / R(n);
        R d0 = warp(o, ray, s, e, f0);
        R d1 = warp(o, ray, s, e, f1);
        R w = refinement_weight(o, h0, ray, d0, d1, sun, bottom, ar, sr0, sr1, sv0, sv1);
        V3<R> iL, iT;
        adaptive_interval(o, h0, ray, d0, d1, sun, E, bottom, ar, w, iL, iT, counter);
        rad = rad + vT * iL;
        vT = vT * iT;
      }
    }
    return vmax(rad, R(0));
  }
  // _camera_transmittance :1788-1825
  V3<R> camera_t(R cam_alt, V3<R> ray, R bottom) const {
    R s, e; bool valid, ground;
    segment_from_altitude(cam_alt, ray.y, bottom, s, e, valid, ground);
    V3<R> tr = splat(R(1));
    if (valid) {
      if (ground) {
        tr = splat(R(0));
      } else {
        V3<R> o = v3(R(0), bottom + cam_alt, R(0));
        V3<R> entry = o + ray * s;
        R radius = norm(entry);
        V3<R> radial = entry / mx(radius, R(1));
        R ea = altitude_on_ray(cam_alt, ray.y, s, bottom);
        tr = sample_t(ea, dot(radial, ray), bottom);
      }
    }
    return tr;
  }
};

template <class R>
V3<R> load3(const R* p) { return {p[0], p[1], p[2]}; }
template <class R>
void store3(R* p, V3<R> v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

// ---- kernels -------------------------------------------------------------

// _build_transmittance :1034-1063
template <class R>
void build_transmittance(const AtmParams& P, R bottom, R* out) {
  Model<R> m(P);
  const int W = P.transmittance_lut_width, H = P.transmittance_lut_height;
#pragma omp parallel for schedule(dynamic, 16)
  for (int idx = 0; idx < W * H; ++idx) {
    int x = idx / H, y = idx % H;
    R u = (R(x) + R(0.5)) / R(W);
    R v = (R(y) + R(0.5)) / R(H);
    R h, c, d;
    m.t_uv_to_ray(u, v, bottom, h, c, d);
    R s = m_sqrt(mx(R(1) - c * c, R(0)));
    R radius = bottom + h;
    V3<R> o = v3(R(0), radius, R(0));
    V3<R> ray = v3(s, c, R(0));
    V3<R> tr = m.integrate_extinction(o, ray, R(0), d, bottom);
    store3(out + static_cast<size_t>(idx) * 3, vclamp(tr, R(0), R(1)));
  }
}

// _build_multi_scattering :1065-1206
template <class R>
void build_multi_scattering(const AtmParams& P, R bottom, const R* E3, R ar, const R* tlut, R* out, int64_t* samples) {
  Model<R> m(P);
  m.tlut = {tlut, P.transmittance_lut_width, P.transmittance_lut_height};
  const V3<R> E = load3(E3);
  const int W = P.multi_scattering_lut_width, H = P.multi_scattering_lut_height;
  const int ndir = P.multi_scattering_directions, nstep = P.multi_scattering_steps;
  int64_t count = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : count)
  for (int idx = 0; idx < W * H; ++idx) {
    int x = idx / H, y = idx % H;
    R u = (R(x) + R(0.5)) / R(W);
    R v = (R(y) + R(0.5)) / R(H);
    R h0 = v * v * m.top();
    R radius = bottom + h0;
    R sc = m.sun_u_to_cosine(u, h0, bottom);
    R ss = m_sqrt(mx(R(1) - sc * sc, R(0)));
    V3<R> sun = v3(ss, sc, R(0));
    V3<R> o = v3(R(0), radius, R(0));
    V3<R> Lsum = splat(R(0)), Fsum = splat(R(0));
    for (int di = 0; di < ndir; ++di) {
      R si = R(di) + R(0.5);
      R dc = R(1) - R(2) * si / R(ndir);
      R ds = m_sqrt(mx(R(1) - dc * dc, R(0)));
      R az = R(di) * R(2.39996323);
      V3<R> ray = v3(ds * m_cos(az), dc, ds * m_sin(az));
      R s, e; bool valid, ground;
      m.segment_vec(o, ray, bottom, s, e, valid, ground);
      V3<R> dL = splat(R(0)), dF = splat(R(0)), pT = splat(R(1));
      if (valid) {
        for (int pi = 0; pi < nstep; ++pi) {
          R f0 = R(pi) / R(nstep);
          R f1 = R(pi + 1) / R(nstep);
          R d0 = m.warp(o, ray, s, e, f0);
          R d1 = m.warp(o, ray, s, e, f1);
          R dist = (d0 + d1) * R(0.5);
          R step = d1 - d0;
          V3<R> point = o + ray * dist;
          R hh = m.altitude_on_ray(h0, dc, dist, bottom);
          V3<R> ext = m.extinction(hh);
          V3<R> sT, sI;
          m.segment_integral(ext, step, sT, sI);
          V3<R> src = m.scattering_source(point, hh, ray, sun, E, bottom, ar, false);
          dL = dL + pT * src * sI;
          dF = dF + pT * m.scattering(hh) * sI;
          pT = pT * sT;
          ++count;
        }
        if (ground) {
          V3<R> gp = o + ray * e;
          V3<R> gn = gp * (R(1) / norm(gp));  // normalized()
          R gsc = dot(gn, sun);
          V3<R> gT = m.sample_solar_t(R(0), gsc, bottom, ar);
          V3<R> gL = m.albedo() * E * gT * mx(gsc, R(0)) / R(kPi);
          dL = dL + pT * gL;
        }
      }
      Lsum = Lsum + dL;
      Fsum = Fsum + dF;
    }
    V3<R> avgL = Lsum / R(ndir);
    V3<R> avgF = vclamp(Fsum / R(ndir), R(0), R(0.95));
    store3(out + static_cast<size_t>(idx) * 3, vmax(avgL / (splat(R(1)) - avgF), R(0)));
  }
  if (samples) *samples = count;
}

// _build_sky_view :1208-1302
template <class R>
void build_sky_view(const AtmParams& P, R bottom, R cam_alt, R sun_cos, const R* E3, R ar, const R* tlut, const R* mslut,
                    R* out) {
  Model<R> m(P);
  m.tlut = {tlut, P.transmittance_lut_width, P.transmittance_lut_height};
  m.mslut = {mslut, P.multi_scattering_lut_width, P.multi_scattering_lut_height};
  const V3<R> E = load3(E3);
  const int W = P.sky_view_lut_width, H = P.sky_view_lut_height, n = P.sky_view_steps;
  R ss = m_sqrt(mx(R(1) - sun_cos * sun_cos, R(0)));
  V3<R> sun = v3(ss, sun_cos, R(0));
  R sh = mx(cam_alt, R(0));
  R sr = bottom + sh;
  V3<R> o = v3(R(0), sr, R(0));
#pragma omp parallel for schedule(dynamic, 8)
  for (int idx = 0; idx < W * H; ++idx) {
    int x = idx / H, y = idx % H;
    R az = (R(x) + R(0.5)) / R(W) * R(kPi);
    R vv = (R(y) + R(0.5)) / R(H);
    R zen = m.sky_v_to_zenith(vv, sh, bottom);
    R vc = m_cos(zen), vs = m_sin(zen);
    V3<R> ray = v3(vs * m_cos(az), vc, vs * m_sin(az));
    R s, e; bool valid, ground;
    m.segment_from_altitude(sh, vc, bottom, s, e, valid, ground);
    V3<R> rad = splat(R(0));
    if (valid) {
      V3<R> vT = splat(R(1));
      for (int i = 0; i < n; ++i) {
        R f0 = R(i) / R(n);
        R f1 = R(i + 1) / R(n);
        R d0 = m.warp(o, ray, s, e, f0);
        R d1 = m.warp(o, ray, s, e, f1);
        R dist = (d0 + d1) * R(0.5);
        R step = d1 - d0;
        V3<R> point = o + ray * dist;
        R hh = m.altitude_on_ray(sh, vc, dist, bottom);
        V3<R> src = m.scattering_source(point, hh, ray, sun, E, bottom, ar, true);
        V3<R> ext = m.extinction(hh);
        V3<R> sT, sI;
        m.segment_integral(ext, step, sT, sI);
        rad = rad + vT * src * sI;
        vT = vT * sT;
      }
    }
    store3(out + static_cast<size_t>(idx) * 3, vmax(rad, R(0)));
  }
}

// _build_aerial_perspective :1304-1420
template <class R>
void build_aerial(const AtmParams& P, int width, int height, R bottom, R cam_alt, const R* sun3, const R* E3, R ar,
                  const R* right3, const R* up3, const R* fwd3, R tanfov, const R* tlut, const R* mslut, R* out) {
  Model<R> m(P);
  m.tlut = {tlut, P.transmittance_lut_width, P.transmittance_lut_height};
  m.mslut = {mslut, P.multi_scattering_lut_width, P.multi_scattering_lut_height};
  const V3<R> sun = load3(sun3), E = load3(E3), right = load3(right3), up = load3(up3), fwd = load3(fwd3);
  const int AW = P.aerial_lut_width, AH = P.aerial_lut_height, AD = P.aerial_lut_depth, ns = P.aerial_steps_per_slice;
  R aspect = R(width) / R(height);
  V3<R> o = v3(R(0), bottom + cam_alt, R(0));
#pragma omp parallel for schedule(dynamic, 1)
  for (int idx = 0; idx < AW * AH; ++idx) {
    int x = idx / AH, y = idx % AH;
    R u = (R(x) + R(0.5)) / R(AW);
    R v = (R(y) + R(0.5)) / R(AH);
    R sx = (u * R(2) - R(1)) * aspect;
    R sy = v * R(2) - R(1);
    V3<R> rv = (right * sx + up * sy) + fwd / tanfov;
    V3<R> ray = rv * (R(1) / norm(rv));  // Taichi normalized(): v * (1/|v|)
    R as, ae; bool valid;
    m.aerial_prefix(cam_alt, ray.y, bottom, as, ae, valid);
    V3<R> cL = splat(R(0)), cT = splat(R(1));
    R prev = as;
    for (int di = 0; di < AD; ++di) {
      R df = R(di) / R(AD - 1);
      R target = as + (ae - as) * df;
      if (valid) {
        R is = mx(prev, as);
        R ie = mn(target, ae);
        if (ie > is) {
          for (int k = 0; k < ns; ++k) {
            R f0 = R(k) / R(ns);
            R f1 = R(k + 1) / R(ns);
            R d0 = m.warp(o, ray, is, ie, f0);
            R d1 = m.warp(o, ray, is, ie, f1);
            R dist = (d0 + d1) * R(0.5);
            R step = d1 - d0;
            V3<R> point = o + ray * dist;
            R hh = m.altitude_on_ray(cam_alt, ray.y, dist, bottom);
            V3<R> ext = m.extinction(hh);
            V3<R> sT, sI;
            m.segment_integral(ext, step, sT, sI);
            V3<R> src = m.scattering_source(point, hh, ray, sun, E, bottom, ar, true);
            cL = cL + cT * src * sI;
            cT = cT * sT;
          }
        }
      }
      store3(out + (static_cast<size_t>(idx) * AD + di) * 3, vmax(cL, R(0)));
      prev = target;
    }
  }
}

// Sky radiance along n arbitrary rays from altitudes h[i]: the march of
// _build_sky_view :1208-1302 for a given direction and sun (per ray).
template <class R>
void sky_rays(const AtmParams& P, R bottom, int n_rays, const R* h, const R* rays, const R* suns, const R* E3, R ar,
              const R* tlut, const R* mslut, R* out) {
  Model<R> m(P);
  m.tlut = {tlut, P.transmittance_lut_width, P.transmittance_lut_height};
  m.mslut = {mslut, P.multi_scattering_lut_width, P.multi_scattering_lut_height};
  const V3<R> E = load3(E3);
  const int n = P.sky_view_steps;
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n_rays; ++i) {
    const R sh = mx(h[i], R(0));
    const V3<R> o = v3(R(0), bottom + sh, R(0));
    const V3<R> ray = load3(rays + 3 * static_cast<size_t>(i)), sun = load3(suns + 3 * static_cast<size_t>(i));
    R s, e; bool valid, ground;
    m.segment_from_altitude(sh, ray.y, bottom, s, e, valid, ground);
    V3<R> rad = splat(R(0));
    if (valid) {
      V3<R> vT = splat(R(1));
      for (int k = 0; k < n; ++k) {
        R d0 = m.warp(o, ray, s, e, R(k) / R(n));
        R d1 = m.warp(o, ray, s, e, R(k + 1) / R(n));
        R dist = (d0 + d1) * R(0.5);
        R step = d1 - d0;
        R hh = m.altitude_on_ray(sh, ray.y, dist, bottom);
        V3<R> src = m.scattering_source(o + ray * dist, hh, ray, sun, E, bottom, ar, true);
        V3<R> sT, sI;
        m.segment_integral(m.extinction(hh), step, sT, sI);
        rad = rad + vT * src * sI;
        vT = vT * sT;
      }
    }
    store3(out + 3 * static_cast<size_t>(i), vmax(rad, R(0)));
  }
}

// Camera-to-surface in-scattering and transmittance of n rays from
// altitudes h[i] to surface distances sd[i]: _surface_aerial_scattering
// :1757-1786 and _surface_segment_transmittance :1603-1665.
template <class R>
void surface_rays(const AtmParams& P, R bottom, int n_rays, const R* h, const R* rays, const R* sd, const R* suns,
                  const R* E3, R ar, const R* tlut, const R* mslut, R* out_L, R* out_T) {
  Model<R> m(P);
  m.tlut = {tlut, P.transmittance_lut_width, P.transmittance_lut_height};
  m.mslut = {mslut, P.multi_scattering_lut_width, P.multi_scattering_lut_height};
  const V3<R> E = load3(E3);
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n_rays; ++i) {
    const R sh = mx(h[i], R(0));
    const V3<R> o = v3(R(0), bottom + sh, R(0));
    const V3<R> ray = load3(rays + 3 * static_cast<size_t>(i)), sun = load3(suns + 3 * static_cast<size_t>(i));
    store3(out_L + 3 * static_cast<size_t>(i), m.integrate_surface(o, sh, ray, sd[i], sun, E, bottom, ar, nullptr));
    store3(out_T + 3 * static_cast<size_t>(i), m.surface_segment_t(o, sh, ray, sd[i], bottom));
  }
}

struct Image {
  int stride_x, stride_y, channels;
  size_t off(int x, int y) const { return (static_cast<size_t>(x) * stride_x + static_cast<size_t>(y) * stride_y) * channels; }
};

// _prepare_surface_lighting :1422-1472
template <class R>
void prepare_surface(const AtmParams& P, int W, int H, const R* pos, const int32_t* sid, Image img, R bottom,
                     R cam_alt, const R* sun3, R ar, const R* right3, const R* up3, const R* fwd3, const R* tlut,
                     const R* mslut, R* out_sun_t, R* out_sky) {
  Model<R> m(P);
  m.tlut = {tlut, P.transmittance_lut_width, P.transmittance_lut_height};
  m.mslut = {mslut, P.multi_scattering_lut_width, P.multi_scattering_lut_height};
  const V3<R> sun = load3(sun3), right = load3(right3), up = load3(up3), fwd = load3(fwd3);
  V3<R> cpp = v3(R(0), bottom + cam_alt, R(0));
#pragma omp parallel for schedule(dynamic, 64)
  for (int idx = 0; idx < W * H; ++idx) {
    int x = idx / H, y = idx % H;
    size_t o = img.off(x, y);
    size_t oi = static_cast<size_t>(x) * img.stride_x + static_cast<size_t>(y) * img.stride_y;
    V3<R> sT = splat(R(1)), sky = splat(R(0));
    if (sid[oi] >= 0) {
      V3<R> vp = load3(pos + o);
      V3<R> lp = (right * vp.x + up * vp.y) + fwd * vp.z;
      V3<R> pp = cpp + lp;
      R radius = norm(pp);
      V3<R> radial = pp / mx(radius, R(1));
      R sd = norm(lp);
      V3<R> lr = lp / mx(sd, R(1));
      R h = m.altitude_on_ray(cam_alt, lr.y, sd, bottom);
      R sc = dot(radial, sun);
      sT = m.sample_solar_t(h, sc, bottom, ar);
      sky = m.sample_ms(h, sc, bottom);
    }
    store3(out_sun_t + o, sT);
    store3(out_sky + o, vmax(sky, R(0)));
  }
}

// _composite :1827-2055, one pixel
template <class R>
V3<R> composite_pixel(const Model<R>& m, const CompositeArgs& A, int px, int py, V3<R> scene, V3<R> space,
                      int32_t sid, V3<R> pos, int64_t* counter) {
  const R bottom = R(A.bottom), cam_alt = R(A.cam_alt), sky_alt = R(A.sky_alt), ar = R(A.ar), tanfov = R(A.tanfov);
  const V3<R> sun = v3(R(A.sun[0]), R(A.sun[1]), R(A.sun[2]));
  const V3<R> E = v3(R(A.E[0]), R(A.E[1]), R(A.E[2]));
  const V3<R> disk = v3(R(A.disk[0]), R(A.disk[1]), R(A.disk[2]));
  const V3<R> right = v3(R(A.right[0]), R(A.right[1]), R(A.right[2]));
  const V3<R> up = v3(R(A.up[0]), R(A.up[1]), R(A.up[2]));
  const V3<R> fwd = v3(R(A.fwd[0]), R(A.fwd[1]), R(A.fwd[2]));
  const int W = A.width, H = A.height;
  R aspect = R(W) / R(H);
  V3<R> color = scene;
  R su = (R(px) + R(0.5)) / R(W);
  R sv = (R(py) + R(0.5)) / R(H);
  R sx = (su * R(2) - R(1)) * aspect;
  R sy = sv * R(2) - R(1);
  V3<R> rv = (right * sx + up * sy) + fwd / tanfov;
  V3<R> ray = rv * (R(1) / norm(rv));  // Taichi normalized(): v * (1/|v|)
  V3<R> origin = v3(R(0), bottom + cam_alt, R(0));
  const int view = A.diagnostic_view;
  if (view == ATM_VIEW_COMPOSITE) {
    if (sid >= 0) {
      R sd = norm(pos);
      V3<R> scat = m.integrate_surface(origin, cam_alt, ray, sd, sun, E, bottom, ar, counter);
      V3<R> tr = m.surface_segment_t(origin, cam_alt, ray, sd, bottom);
      color = scat + color * tr;
    } else {
      V3<R> tr = m.camera_t(cam_alt, ray, bottom);
      V3<R> sky = m.sample_sky_view(ray, sun, sky_alt, bottom);
      V3<R> star = space * tr;
      const V3<R> lw = v3(R(0.2126), R(0.7152), R(0.0722));
      R skyl = dot(sky, lw);
      R starl = dot(star, lw);
      R contrast = starl / mx(skyl, R(1.0e-5));
      R vis = clampr((contrast - R(A.star_start)) / mx(R(A.star_end) - R(A.star_start), R(1.0e-5)), R(0), R(1));
      vis = vis * vis * (R(3) - R(2) * vis);
      color = (sky + color * tr) + star * vis;
      R ad = m_acos(clampr(dot(ray, sun), R(-1), R(1)));
      R pf = m_atan2(tanfov * R(1.41421356) / R(H), R(1));
      R cov = clampr((ar + pf - ad) / mx(R(2) * pf, R(1.0e-8)), R(0), R(1));
      cov = cov * cov * (R(3) - R(2) * cov);
      color = color + disk * tr * cov;
    }
  } else if (view == ATM_VIEW_SKY_VIEW) {
    color = m.sample_sky_view(ray, sun, sky_alt, bottom);
  } else if (view == ATM_VIEW_CAMERA_TRANSMITTANCE) {
    color = m.camera_t(cam_alt, ray, bottom);
  } else if (view == ATM_VIEW_TRANSMITTANCE_LUT) {
    int lx = std::min(static_cast<int>(su * R(m.tlut.w)), m.tlut.w - 1);
    int ly = std::min(static_cast<int>(sv * R(m.tlut.h)), m.tlut.h - 1);
    color = m.tlut.at(lx, ly);
  } else if (view == ATM_VIEW_MULTI_SCATTERING_LUT) {
    int lx = std::min(static_cast<int>(su * R(m.mslut.w)), m.mslut.w - 1);
    int ly = std::min(static_cast<int>(sv * R(m.mslut.h)), m.mslut.h - 1);
    color = m.mslut.at(lx, ly);
  } else if (view == ATM_VIEW_AERIAL_SCATTERING || view == ATM_VIEW_AERIAL_DIRECT_ONLY) {
    color = splat(R(0));
    if (sid >= 0) color = m.integrate_surface(origin, cam_alt, ray, norm(pos), sun, E, bottom, ar, counter);
  } else if (view == ATM_VIEW_AERIAL_FROXEL_ONLY) {
    color = splat(R(0));
    if (sid >= 0) color = m.sample_aerial_scattering(su, sv, norm(pos), cam_alt, ray, bottom);
  } else if (view == ATM_VIEW_AERIAL_BLEND_WEIGHT) {
    R w = sid >= 0 ? R(1) : R(0);
    color = splat(w);
  } else if (view == ATM_VIEW_AERIAL_TRANSMITTANCE) {
    color = splat(R(0));
    if (sid >= 0) color = m.surface_segment_t(origin, cam_alt, ray, norm(pos), bottom);
  } else {
    R mask = sid >= 0 ? R(1) : R(0);
    color = splat(mask);
  }
  return vmax(color, R(0));
}

template <class R>
int64_t composite(const AtmParams& P, const CompositeArgs& A, Image img, const R* scene, const R* space,
                  const int32_t* sid, const R* pos, const R* tlut, const R* mslut, const R* svlut, const R* aplut,
                  R* hdr, const int32_t* pixel_list, int64_t n_list, double* margin) {
  Model<R> m(P);
  m.tlut = {tlut, P.transmittance_lut_width, P.transmittance_lut_height};
  m.mslut = {mslut, P.multi_scattering_lut_width, P.multi_scattering_lut_height};
  m.svlut = {svlut, P.sky_view_lut_width, P.sky_view_lut_height};
  m.aplut = {aplut, P.aerial_lut_width, P.aerial_lut_height, P.aerial_lut_depth};
  const int64_t total = pixel_list ? n_list : static_cast<int64_t>(A.width) * A.height;
  int64_t count = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : count)
  for (int64_t k = 0; k < total; ++k) {
    int64_t pix = pixel_list ? pixel_list[k] : k;
    int x = static_cast<int>(pix / A.height), y = static_cast<int>(pix % A.height);
    size_t o = img.off(x, y);
    size_t oi = static_cast<size_t>(x) * img.stride_x + static_cast<size_t>(y) * img.stride_y;
    int64_t local = 0;
    g_cutoff_margin = HUGE_VAL;
    V3<R> c = composite_pixel(m, A, x, y, load3(scene + o), load3(space + o), sid[oi], load3(pos + o), &local);
    store3(hdr + o, c);
    if (margin) margin[oi] = g_cutoff_margin;
    count += local;
  }
  return count;
}

}  // namespace


// ---- operation counting --------------------------------------------------
// CountF behaves as float and counts every arithmetic operation the
// restatement performs: the algorithmic operation count of the reference's
// kernels (comparisons, min/max and clamps are not counted).  Counters are
// per thread; counting runs use one thread.
namespace opcount {
enum { kAdd, kMul, kDiv, kSqrt, kExp, kAcos, kCosSin, kPow, kAtan2, kN };
thread_local uint64_t counts[kN];
struct CountF {
  float v;
  CountF() = default;
  constexpr CountF(double x) : v(float(x)) {}
  explicit operator int() const { return int(v); }
};
inline CountF mkc(float x) { CountF r; r.v = x; return r; }
inline CountF operator+(CountF a, CountF b) { ++counts[kAdd]; return mkc(a.v + b.v); }
inline CountF operator-(CountF a, CountF b) { ++counts[kAdd]; return mkc(a.v - b.v); }
inline CountF operator-(CountF a) { return mkc(-a.v); }
inline CountF operator*(CountF a, CountF b) { ++counts[kMul]; return mkc(a.v * b.v); }
inline CountF operator/(CountF a, CountF b) { ++counts[kDiv]; return mkc(a.v / b.v); }
inline bool operator<(CountF a, CountF b) { return a.v < b.v; }
inline bool operator>(CountF a, CountF b) { return a.v > b.v; }
inline bool operator<=(CountF a, CountF b) { return a.v <= b.v; }
inline bool operator>=(CountF a, CountF b) { return a.v >= b.v; }
inline double as_d(CountF x) { return double(x.v); }
inline CountF sqrt(CountF x) { ++counts[kSqrt]; return mkc(std::sqrt(x.v)); }
inline CountF exp(CountF x) { ++counts[kExp]; return mkc(std::exp(x.v)); }
inline CountF acos(CountF x) { ++counts[kAcos]; return mkc(std::acos(x.v)); }
inline CountF cos(CountF x) { ++counts[kCosSin]; return mkc(std::cos(x.v)); }
inline CountF sin(CountF x) { ++counts[kCosSin]; return mkc(std::sin(x.v)); }
inline CountF pow(CountF x, CountF y) { ++counts[kPow]; return mkc(std::pow(x.v, y.v)); }
inline CountF atan2(CountF y, CountF x) { ++counts[kAtan2]; return mkc(std::atan2(y.v, x.v)); }
inline CountF fabs(CountF x) { return mkc(std::fabs(x.v)); }
inline CountF floor(CountF x) { return mkc(std::floor(x.v)); }
static_assert(sizeof(CountF) == sizeof(float), "CountF must alias float buffers");
}  // namespace opcount

// ---- C entry points for ctypes -------------------------------------------
#define ORC_EXPORT extern "C" __attribute__((visibility("default")))

#define ORC_DEFINE(SUFFIX, R)                                                                                        \
  ORC_EXPORT void orc_build_transmittance_##SUFFIX(const AtmParams* p, double bottom, R* out) {                      \
    build_transmittance<R>(*p, R(bottom), out);                                                                      \
  }                                                                                                                  \
  ORC_EXPORT int64_t orc_build_multi_scattering_##SUFFIX(const AtmParams* p, double bottom, const double* E,         \
                                                         double ar, const R* tlut, R* out) {                         \
    R e[3] = {R(E[0]), R(E[1]), R(E[2])};                                                                            \
    int64_t n = 0;                                                                                                   \
    build_multi_scattering<R>(*p, R(bottom), e, R(ar), tlut, out, &n);                                               \
    return n;                                                                                                        \
  }                                                                                                                  \
  ORC_EXPORT void orc_build_sky_view_##SUFFIX(const AtmParams* p, double bottom, double cam_alt, double sun_cos,     \
                                              const double* E, double ar, const R* tlut, const R* mslut, R* out) {   \
    R e[3] = {R(E[0]), R(E[1]), R(E[2])};                                                                            \
    build_sky_view<R>(*p, R(bottom), R(cam_alt), R(sun_cos), e, R(ar), tlut, mslut, out);                            \
  }                                                                                                                  \
  ORC_EXPORT void orc_build_aerial_##SUFFIX(const AtmParams* p, int width, int height, double bottom, double cam_alt, \
                                            const double* sun, const double* E, double ar, const double* right,     \
                                            const double* up, const double* fwd, double tanfov, const R* tlut,      \
                                            const R* mslut, R* out) {                                                \
    R s[3] = {R(sun[0]), R(sun[1]), R(sun[2])}, e[3] = {R(E[0]), R(E[1]), R(E[2])};                                  \
    R r[3] = {R(right[0]), R(right[1]), R(right[2])}, u[3] = {R(up[0]), R(up[1]), R(up[2])};                         \
    R f[3] = {R(fwd[0]), R(fwd[1]), R(fwd[2])};                                                                      \
    build_aerial<R>(*p, width, height, R(bottom), R(cam_alt), s, e, R(ar), r, u, f, R(tanfov), tlut, mslut, out);    \
  }                                                                                                                  \
  ORC_EXPORT void orc_prepare_surface_##SUFFIX(const AtmParams* p, int W, int H, int stride_x, int stride_y,         \
                                               int channels, const R* pos, const int32_t* sid, double bottom,       \
                                               double cam_alt, const double* sun, double ar, const double* right,   \
                                               const double* up, const double* fwd, const R* tlut, const R* mslut,  \
                                               R* out_sun_t, R* out_sky) {                                           \
    R s[3] = {R(sun[0]), R(sun[1]), R(sun[2])};                                                                      \
    R r[3] = {R(right[0]), R(right[1]), R(right[2])}, u[3] = {R(up[0]), R(up[1]), R(up[2])};                         \
    R f[3] = {R(fwd[0]), R(fwd[1]), R(fwd[2])};                                                                      \
    prepare_surface<R>(*p, W, H, pos, sid, Image{stride_x, stride_y, channels}, R(bottom), R(cam_alt), s, R(ar), r,  \
                       u, f, tlut, mslut, out_sun_t, out_sky);                                                       \
  }                                                                                                                  \
  ORC_EXPORT void orc_sky_rays_##SUFFIX(const AtmParams* p, double bottom, int n, const R* h, const R* rays,         \
                                        const R* suns, const double* E, double ar, const R* tlut, const R* mslut,   \
                                        R* out) {                                                                    \
    R e[3] = {R(E[0]), R(E[1]), R(E[2])};                                                                            \
    sky_rays<R>(*p, R(bottom), n, h, rays, suns, e, R(ar), tlut, mslut, out);                                        \
  }                                                                                                                  \
  ORC_EXPORT void orc_surface_rays_##SUFFIX(const AtmParams* p, double bottom, int n, const R* h, const R* rays,     \
                                            const R* sd, const R* suns, const double* E, double ar, const R* tlut,  \
                                            const R* mslut, R* out_L, R* out_T) {                                    \
    R e[3] = {R(E[0]), R(E[1]), R(E[2])};                                                                            \
    surface_rays<R>(*p, R(bottom), n, h, rays, sd, suns, e, R(ar), tlut, mslut, out_L, out_T);                       \
  }                                                                                                                  \
  ORC_EXPORT int64_t orc_composite_##SUFFIX(                                                                         \
      const AtmParams* p, const CompositeArgs* a, int stride_x, int stride_y, int channels, const R* scene,           \
      const R* space, const int32_t* sid, const R* pos, const R* tlut, const R* mslut, const R* svlut,               \
      const R* aplut, R* hdr, const int32_t* pixel_list, int64_t n_list, double* margin) {                           \
    return composite<R>(*p, *a, Image{stride_x, stride_y, channels}, scene, space, sid, pos, tlut, mslut, svlut,     \
                        aplut, hdr, pixel_list, n_list, margin);                                                     \
  }

ORC_DEFINE(f32, float)
ORC_DEFINE(f64, double)
ORC_DEFINE(cnt, opcount::CountF)

// Operation counts of the calling thread since the last reset: add/sub, mul,
// div, sqrt, exp, acos, cos+sin, pow, atan2.
ORC_EXPORT void orc_op_counts(uint64_t out[9], int reset) {
  for (int i = 0; i < opcount::kN; ++i) {
    out[i] = opcount::counts[i];
    if (reset) opcount::counts[i] = 0;
  }
}

ORC_EXPORT void orc_set_series_weight(int on) { g_series_weight = on; }

ORC_EXPORT int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

ORC_EXPORT void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
