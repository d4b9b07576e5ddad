// atm_capi.cu - C ABI of libplanet_atm (declared in include/atm_capi.h).
//
// Host side of the reference's AtmosphereRenderer (atmosphere/renderer.py
// :51-116, :2057-2238): the renderer state, the LUT cache keys and the
// float rounding points of update / prepare_frame / composite live here, in
// native code, so a non-Python host gets the same behaviour as the Python
// layer (which is a thin ctypes wrapper over these functions).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "atm_capi.h"
#include "atm_kernels.h"

#define ATM_API extern "C" __attribute__((visibility("default")))

namespace {

thread_local std::string g_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(ATM_E_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define ATM_CUDA(call, what)                  \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

constexpr double kPi = 3.141592653589793;

bool finite_nonneg3(const double* v) {
  for (int i = 0; i < 3; ++i)
    if (!std::isfinite(v[i]) || v[i] < 0.0) return false;
  return true;
}

// Validation ranges of the reference AtmosphereConfig (config.py:61-128).
int validate(const AtmParams& p) {
  if (!finite_nonneg3(p.rayleigh_scattering_per_m) || !finite_nonneg3(p.mie_scattering_per_m) ||
      !finite_nonneg3(p.mie_extinction_per_m) || !finite_nonneg3(p.absorption_extinction_per_m) ||
      !finite_nonneg3(p.ground_albedo))
    return fail(ATM_E_INVALID, "atmosphere coefficients must contain three non-negative values");
  for (double a : p.ground_albedo)
    if (a > 1.0) return fail(ATM_E_INVALID, "atmosphere.ground_albedo must remain in [0, 1]");
  const double positive[] = {p.top_altitude_m, p.rayleigh_scale_height_m, p.mie_scale_height_m,
                             p.absorption_half_width_m};
  for (double v : positive)
    if (!std::isfinite(v) || v <= 0.0) return fail(ATM_E_INVALID, "atmosphere lengths must be positive and finite");
  if (!(0.0 <= p.absorption_peak_altitude_m && p.absorption_peak_altitude_m <= p.top_altitude_m))
    return fail(ATM_E_INVALID, "atmosphere absorption peak must lie inside the shell");
  if (!(-0.99 < p.mie_phase_g && p.mie_phase_g < 0.99))
    return fail(ATM_E_INVALID, "atmosphere.mie_phase_g must be in (-0.99, 0.99)");
  for (int i = 0; i < 3; ++i)
    if (p.mie_scattering_per_m[i] > p.mie_extinction_per_m[i])
      return fail(ATM_E_INVALID, "Mie scattering cannot exceed Mie extinction");
  struct Range {
    int32_t v, lo, hi;
    const char* name;
  } ranges[] = {
      {p.transmittance_lut_width, 16, 2048, "transmittance_lut_width"},
      {p.transmittance_lut_height, 16, 1024, "transmittance_lut_height"},
      {p.sky_view_lut_width, 16, 2048, "sky_view_lut_width"},
      {p.sky_view_lut_height, 16, 2048, "sky_view_lut_height"},
      {p.multi_scattering_lut_width, 8, 256, "multi_scattering_lut_width"},
      {p.multi_scattering_lut_height, 8, 256, "multi_scattering_lut_height"},
      {p.aerial_lut_width, 4, 256, "aerial_lut_width"},
      {p.aerial_lut_height, 4, 256, "aerial_lut_height"},
      {p.aerial_lut_depth, 8, 256, "aerial_lut_depth"},
      {p.transmittance_steps, 4, 256, "transmittance_steps"},
      {p.multi_scattering_directions, 4, 128, "multi_scattering_directions"},
      {p.multi_scattering_steps, 4, 128, "multi_scattering_steps"},
      {p.sky_view_steps, 4, 256, "sky_view_steps"},
      {p.aerial_steps_per_slice, 1, 16, "aerial_steps_per_slice"},
      {p.aerial_horizon_raymarch_steps, 4, 64, "aerial_horizon_raymarch_steps"},
      {p.aerial_terminator_substeps, 2, 16, "aerial_terminator_substeps"},
  };
  for (const Range& r : ranges)
    if (r.v < r.lo || r.v > r.hi) return fail(ATM_E_INVALID, "%s must be in %d..%d", r.name, r.lo, r.hi);
  return ATM_OK;
}

// math.radians: x * (pi / 180) in double, then the kernel argument's f32 rounding
float radians_f32(double degrees) { return float(degrees * (kPi / 180.0)); }

}  // namespace

namespace atm {

DevParams make_dev_params(const AtmParams& p) {
  DevParams d{};
  d.top = float(p.top_altitude_m);
  for (int i = 0; i < 3; ++i) {
    d.beta_r[i] = float(p.rayleigh_scattering_per_m[i]);
    d.beta_ms[i] = float(p.mie_scattering_per_m[i]);
    d.beta_me[i] = float(p.mie_extinction_per_m[i]);
    d.beta_o[i] = float(p.absorption_extinction_per_m[i]);
    d.albedo[i] = float(p.ground_albedo[i]);
  }
  d.h_r = float(p.rayleigh_scale_height_m);
  d.h_m = float(p.mie_scale_height_m);
  d.oz_peak = float(p.absorption_peak_altitude_m);
  d.oz_half = float(p.absorption_half_width_m);
  const double g = p.mie_phase_g;  // Python-constant folding in double (renderer.py:795-804)
  d.mie_c1 = float(1.0 + g * g);
  d.mie_c2 = float(2.0 * g);
  d.mie_k1 = float(3.0 * (1.0 - g * g));
  d.mie_k2 = float(8.0 * kPi * (2.0 + g * g));
  d.ray_k = float(16.0 * kPi);
  d.inv_h_r = float(1.0 / p.rayleigh_scale_height_m);
  d.inv_h_m = float(1.0 / p.mie_scale_height_m);
  d.inv_oz_half = float(1.0 / p.absorption_half_width_m);
  d.inv_top = float(1.0 / p.top_altitude_m);
  d.t_w = p.transmittance_lut_width;
  d.t_h = p.transmittance_lut_height;
  d.ms_w = p.multi_scattering_lut_width;
  d.ms_h = p.multi_scattering_lut_height;
  d.sv_w = p.sky_view_lut_width;
  d.sv_h = p.sky_view_lut_height;
  d.ap_w = p.aerial_lut_width;
  d.ap_h = p.aerial_lut_height;
  d.ap_d = p.aerial_lut_depth;
  d.t_steps = p.transmittance_steps;
  d.ms_dirs = p.multi_scattering_directions;
  d.ms_steps = p.multi_scattering_steps;
  d.sv_steps = p.sky_view_steps;
  d.ap_steps = p.aerial_steps_per_slice;
  d.limb_steps = p.aerial_horizon_raymarch_steps;
  d.substeps = p.aerial_terminator_substeps;
  return d;
}

}  // namespace atm

struct AtmHandle {
  AtmParams params;
  atm::DevParams dev;
  int32_t width = 0, height = 0;
  float4* lut[4] = {nullptr, nullptr, nullptr, nullptr};
  int32_t dims[4][3] = {};
  unsigned long long* samples = nullptr;
  // cache keys (reference renderer.py:97-107); valid flags stand for "not None"
  bool t_valid = false;
  double t_key = 0.0;
  bool ms_valid = false;
  double ms_key[5] = {};  // R, E[3], angular radius (f32-rounded)
  bool sky_valid = false;
  double sky_key[6] = {};  // altitude, sun cosine, E[3], angular radius
  bool aerial_available = false;
  AtmState state{};
  // surrogate composite: fallback queue (4 header words: entries, ticket,
  // timeout flag, padding; then width * height entries)
  uint32_t* queue = nullptr;
  float* calib_lm = nullptr;     // the surrogate calibration's scratch image (width x height x 3)
  float* calib_tiles = nullptr;  // its tile sums, sized for the smallest tile (16 pixels)
  uint8_t* calib_mask = nullptr; // the sky-pixel workload's network-pixel mask (width x height bytes)
  int sm_count = 0;
};

namespace {

size_t lut_texels(const AtmHandle* h, int kind) {
  return size_t(h->dims[kind][0]) * h->dims[kind][1] * h->dims[kind][2];
}

int check_handle(const AtmHandle* h) {
  if (h == nullptr) return fail(ATM_E_INVALID, "null AtmHandle");
  return ATM_OK;
}

int check_image(const AtmHandle* h, const AtmImage* img) {
  if (img == nullptr) return fail(ATM_E_INVALID, "null AtmImage");
  if (img->width != h->width || img->height != h->height)
    return fail(ATM_E_INVALID, "image is %dx%d but the renderer was created for %dx%d", img->width, img->height,
                h->width, h->height);
  if (img->channels != 3 && img->channels != 4) return fail(ATM_E_INVALID, "channels must be 3 or 4");
  if (img->stride_x <= 0 || img->stride_y <= 0) return fail(ATM_E_INVALID, "image strides must be positive");
  return ATM_OK;
}

atm::ImageLayout layout_of(const AtmImage* img) {
  return {img->width, img->height, img->stride_x, img->stride_y, img->channels};
}

void to_f32(const double* in, float* out, int n) {
  for (int i = 0; i < n; ++i) out[i] = float(in[i]);
}

int build_transmittance(AtmHandle* h, double R, cudaStream_t s) {
  ATM_CUDA(atm::launch_transmittance(h->dev, float(R), h->lut[ATM_LUT_TRANSMITTANCE], s), "transmittance build");
  return ATM_OK;
}

int build_multi_scattering(AtmHandle* h, double R, const double E[3], double ar, cudaStream_t s) {
  float e[3];
  to_f32(E, e, 3);
  ATM_CUDA(atm::launch_multi_scattering(h->dev, float(R), e, float(ar), h->lut[ATM_LUT_TRANSMITTANCE],
                                        h->lut[ATM_LUT_MULTI_SCATTERING], h->samples, s),
           "multi-scattering build");
  return ATM_OK;
}

int build_sky_view(AtmHandle* h, double R, double alt, double sun_cos, const double E[3], double ar,
                   cudaStream_t s) {
  float e[3];
  to_f32(E, e, 3);
  ATM_CUDA(atm::launch_sky_view(h->dev, float(R), float(alt), float(sun_cos), e, float(ar),
                                h->lut[ATM_LUT_TRANSMITTANCE], h->lut[ATM_LUT_MULTI_SCATTERING],
                                h->lut[ATM_LUT_SKY_VIEW], h->samples, s),
           "sky-view build");
  return ATM_OK;
}

int build_aerial(AtmHandle* h, int width, int height, double R, double alt, const double sun[3], const double E[3],
                 double ar, const double basis[9], double tanfov, cudaStream_t s) {
  float sn[3], e[3], b[9];
  to_f32(sun, sn, 3);
  to_f32(E, e, 3);
  to_f32(basis, b, 9);
  ATM_CUDA(atm::launch_aerial(h->dev, width, height, float(R), float(alt), sn, e, float(ar), b, b + 3, b + 6,
                              float(tanfov), h->lut[ATM_LUT_TRANSMITTANCE], h->lut[ATM_LUT_MULTI_SCATTERING],
                              h->lut[ATM_LUT_AERIAL], h->samples, s),
           "aerial-perspective build");
  return ATM_OK;
}

bool finite_n(const double* v, int n) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

}  // namespace

ATM_API const char* atm_last_error(void) { return g_error.c_str(); }

ATM_API int atm_create(const AtmParams* params, int32_t width, int32_t height, AtmHandle** out) {
  if (params == nullptr || out == nullptr) return fail(ATM_E_INVALID, "null argument to atm_create");
  *out = nullptr;
  if (width < 1 || height < 1 || width > 16384 || height > 16384)
    return fail(ATM_E_INVALID, "frame size %dx%d outside 1..16384", width, height);
  int rc = validate(*params);
  if (rc != ATM_OK) return rc;
  AtmHandle* h = new (std::nothrow) AtmHandle();
  if (h == nullptr) return fail(ATM_E_NOMEM, "host allocation failed");
  h->params = *params;
  h->dev = atm::make_dev_params(*params);
  h->width = width;
  h->height = height;
  const int32_t dims[4][3] = {
      {params->transmittance_lut_width, params->transmittance_lut_height, 1},
      {params->multi_scattering_lut_width, params->multi_scattering_lut_height, 1},
      {params->sky_view_lut_width, params->sky_view_lut_height, 1},
      {params->aerial_lut_width, params->aerial_lut_height, params->aerial_lut_depth},
  };
  std::memcpy(h->dims, dims, sizeof(dims));
  for (int k = 0; k < 4; ++k) {
    const size_t bytes = lut_texels(h, k) * sizeof(float4);
    cudaError_t e = cudaMalloc(&h->lut[k], bytes);
    if (e == cudaSuccess) e = cudaMemset(h->lut[k], 0, bytes);
    if (e != cudaSuccess) {
      atm_destroy(h);
      return e == cudaErrorMemoryAllocation ? fail(ATM_E_NOMEM, "LUT allocation failed") : cuda_fail(e, "LUT init");
    }
  }
  cudaError_t e = cudaMalloc(&h->samples, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(h->samples, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) {
    atm_destroy(h);
    return cuda_fail(e, "sample counter");
  }
  *out = h;
  return ATM_OK;
}

ATM_API int atm_destroy(AtmHandle* h) {
  if (h == nullptr) return ATM_OK;
  for (float4*& p : h->lut) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  if (h->samples) cudaFree(h->samples);
  if (h->queue) cudaFree(h->queue);
  if (h->calib_lm) cudaFree(h->calib_lm);
  if (h->calib_tiles) cudaFree(h->calib_tiles);
  if (h->calib_mask) cudaFree(h->calib_mask);
  delete h;
  return ATM_OK;
}

ATM_API int atm_set_luts_frozen(AtmHandle* h, int32_t frozen) {
  int rc = check_handle(h);
  if (rc) return rc;
  const bool f = frozen != 0;
  if (h->state.luts_frozen && !f) h->sky_valid = false;  // renderer.py:2068-2069
  h->state.luts_frozen = f ? 1 : 0;
  return ATM_OK;
}

ATM_API int atm_get_state(const AtmHandle* h, AtmState* out) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (out == nullptr) return fail(ATM_E_INVALID, "null AtmState");
  *out = h->state;
  return ATM_OK;
}

ATM_API int atm_update(AtmHandle* h, double planet_radius_m, double camera_radius_m, const double sun_local[3],
                       const double solar_irradiance[3], double sun_angular_radius_degrees, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (sun_local == nullptr || solar_irradiance == nullptr) return fail(ATM_E_INVALID, "null vector argument");
  if (!std::isfinite(planet_radius_m) || planet_radius_m <= 1.0 || !std::isfinite(camera_radius_m) ||
      !finite_n(sun_local, 3) || !finite_n(solar_irradiance, 3) || !std::isfinite(sun_angular_radius_degrees))
    return fail(ATM_E_INVALID, "non-finite update argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double R = planet_radius_m;
  double n = std::sqrt(sun_local[0] * sun_local[0] + sun_local[1] * sun_local[1] + sun_local[2] * sun_local[2]);
  n = n > 1.0e-12 ? n : 1.0e-12;
  const double sun_y = sun_local[1] / n;
  const double ar = double(radians_f32(sun_angular_radius_degrees));  // renderer.py:2086-2088
  if (!h->t_valid || h->t_key != R) {
    if ((rc = build_transmittance(h, R, s))) return rc;
    h->t_valid = true;
    h->t_key = R;
    h->ms_valid = false;
    h->sky_valid = false;
    h->state.transmittance_rebuilds++;
  }
  const double ms_key[5] = {R, solar_irradiance[0], solar_irradiance[1], solar_irradiance[2], ar};
  if (!h->ms_valid || std::memcmp(ms_key, h->ms_key, sizeof(ms_key)) != 0) {
    if ((rc = build_multi_scattering(h, R, solar_irradiance, ar, s))) return rc;
    std::memcpy(h->ms_key, ms_key, sizeof(ms_key));
    h->ms_valid = true;
    h->sky_valid = false;
    h->state.multi_scattering_rebuilds++;
  }
  // altitude kept apart from the Earth-scale radius before it meets f32 (:2112-2118)
  const double alt_key = double(float(std::fmax(camera_radius_m - R, 0.0)));
  const double zen_key = double(float(std::fmin(std::fmax(sun_y, -1.0), 1.0)));
  const double sky_key[6] = {alt_key, zen_key, solar_irradiance[0], solar_irradiance[1], solar_irradiance[2], ar};
  const bool changed = !h->sky_valid || std::memcmp(sky_key, h->sky_key, sizeof(sky_key)) != 0;
  if (changed && (!h->state.luts_frozen || !h->sky_valid)) {
    if ((rc = build_sky_view(h, R, alt_key, zen_key, solar_irradiance, ar, s))) return rc;
    std::memcpy(h->sky_key, sky_key, sizeof(sky_key));
    h->sky_valid = true;
    h->state.has_sky_snapshot = 1;
    h->state.sky_snapshot_altitude_m = alt_key;
    h->state.sky_snapshot_sun_cosine = zen_key;
    h->state.sky_view_rebuilds++;
  }
  return ATM_OK;
}

ATM_API int atm_prepare_frame(AtmHandle* h, const float* position_view, const int32_t* surface_id,
                              const AtmImage* image, double planet_radius_m, double camera_radius_m,
                              const double sun_local[3], const double solar_irradiance[3],
                              double sun_angular_radius_degrees, const double view_basis[9],
                              double tangent_half_fov, float* surface_sun_transmittance, float* surface_sky_radiance,
                              void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = check_image(h, image))) return rc;
  if (!position_view || !surface_id || !surface_sun_transmittance || !surface_sky_radiance || !sun_local ||
      !solar_irradiance || !view_basis)
    return fail(ATM_E_INVALID, "null pointer argument to atm_prepare_frame");
  if (!finite_n(view_basis, 9) || !finite_n(sun_local, 3) || !std::isfinite(tangent_half_fov) ||
      tangent_half_fov <= 0.0)
    return fail(ATM_E_INVALID, "non-finite or non-positive frame argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double R = planet_radius_m;
  const double alt = std::fmax(camera_radius_m - R, 0.0);
  const float ar = radians_f32(sun_angular_radius_degrees);
  float sn[3], b[9];
  to_f32(sun_local, sn, 3);
  to_f32(view_basis, b, 9);
  ATM_CUDA(atm::launch_prepare_surface(h->dev, layout_of(image), position_view, surface_id, float(R), float(alt), sn,
                                       ar, b, b + 3, b + 6, h->lut[ATM_LUT_TRANSMITTANCE],
                                       h->lut[ATM_LUT_MULTI_SCATTERING], surface_sun_transmittance,
                                       surface_sky_radiance, s),
           "surface lighting");
  if (!h->state.luts_frozen || !h->aerial_available) {
    if ((rc = build_aerial(h, h->width, h->height, R, alt, sun_local, solar_irradiance, double(ar), view_basis,
                           tangent_half_fov, s)))
      return rc;
    h->state.has_aerial_snapshot = 1;
    h->state.aerial_snapshot_altitude_m = camera_radius_m - planet_radius_m;
    h->aerial_available = true;
    h->state.aerial_rebuilds++;
  }
  return ATM_OK;
}

namespace {
// Scalar arguments of the composite (renderer.py :2210-2238 rounding points).
atm::CompositeScalars composite_scalars(const AtmHandle* h, double planet_radius_m, double camera_radius_m,
                                        const double sun_local[3], const double solar_irradiance[3],
                                        const double sun_disk_radiance[3], double sun_angular_radius_degrees,
                                        const double view_basis[9], double tangent_half_fov,
                                        double star_contrast_start, double star_contrast_end) {
  const double alt = std::fmax(camera_radius_m - planet_radius_m, 0.0);
  const double sky_alt = h->state.has_sky_snapshot ? h->state.sky_snapshot_altitude_m : alt;  // :2215-2217
  atm::CompositeScalars A{};
  A.bottom = float(planet_radius_m);
  A.cam_alt = float(alt);
  A.sky_alt = float(sky_alt);
  A.ar = radians_f32(sun_angular_radius_degrees);
  A.tanfov = float(tangent_half_fov);
  A.star_start = float(star_contrast_start);
  A.star_end = float(star_contrast_end);
  to_f32(sun_local, A.sun, 3);
  to_f32(solar_irradiance, A.E, 3);
  to_f32(sun_disk_radiance, A.disk, 3);
  to_f32(view_basis, A.right, 3);
  to_f32(view_basis + 3, A.up, 3);
  to_f32(view_basis + 6, A.fwd, 3);
  A.view = ATM_VIEW_COMPOSITE;
  return A;
}
}  // namespace

ATM_API int atm_composite(AtmHandle* h, const float* scene_hdr, const float* space_hdr, const int32_t* surface_id,
                          const float* position_view, float* hdr, const AtmImage* image, double planet_radius_m,
                          double camera_radius_m, const double sun_local[3], const double solar_irradiance[3],
                          const double sun_disk_radiance[3], double sun_angular_radius_degrees,
                          const double view_basis[9], double tangent_half_fov, double star_contrast_start,
                          double star_contrast_end, int32_t diagnostic_view, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = check_image(h, image))) return rc;
  if (!scene_hdr || !space_hdr || !surface_id || !position_view || !hdr || !sun_local || !solar_irradiance ||
      !sun_disk_radiance || !view_basis)
    return fail(ATM_E_INVALID, "null pointer argument to atm_composite");
  if (!finite_n(view_basis, 9) || !finite_n(sun_local, 3) || !std::isfinite(tangent_half_fov) ||
      tangent_half_fov <= 0.0)
    return fail(ATM_E_INVALID, "non-finite or non-positive frame argument");
  atm::CompositeScalars A =
      composite_scalars(h, planet_radius_m, camera_radius_m, sun_local, solar_irradiance, sun_disk_radiance,
                        sun_angular_radius_degrees, view_basis, tangent_half_fov, star_contrast_start,
                        star_contrast_end);
  A.view = diagnostic_view;
  ATM_CUDA(atm::launch_composite(h->dev, layout_of(image), A, scene_hdr, space_hdr, surface_id, position_view,
                                 h->lut[ATM_LUT_TRANSMITTANCE], h->lut[ATM_LUT_MULTI_SCATTERING],
                                 h->lut[ATM_LUT_SKY_VIEW], h->lut[ATM_LUT_AERIAL], hdr, h->samples,
                                 static_cast<cudaStream_t>(stream)),
           "composite");
  return ATM_OK;
}

ATM_API int atm_build_lut(AtmHandle* h, int32_t kind, const AtmBuildArgs* a, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (a == nullptr) return fail(ATM_E_INVALID, "null AtmBuildArgs");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (kind) {
    case ATM_LUT_TRANSMITTANCE:
      return build_transmittance(h, a->planet_radius_m, s);
    case ATM_LUT_MULTI_SCATTERING:
      return build_multi_scattering(h, a->planet_radius_m, a->solar_irradiance, a->sun_angular_radius_rad, s);
    case ATM_LUT_SKY_VIEW:
      return build_sky_view(h, a->planet_radius_m, a->camera_altitude_m, a->sun_zenith_cosine, a->solar_irradiance,
                            a->sun_angular_radius_rad, s);
    case ATM_LUT_AERIAL:
      if (a->frame_width < 1 || a->frame_height < 1) return fail(ATM_E_INVALID, "aerial build needs the frame size");
      return build_aerial(h, a->frame_width, a->frame_height, a->planet_radius_m, a->camera_altitude_m, a->sun_local,
                          a->solar_irradiance, a->sun_angular_radius_rad, a->view_basis, a->tangent_half_fov, s);
    default:
      return fail(ATM_E_INVALID, "unknown LUT kind %d", kind);
  }
}

ATM_API int atm_lut_info(const AtmHandle* h, int32_t kind, int32_t dims[3], void** device_ptr) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (kind < 0 || kind > 3) return fail(ATM_E_INVALID, "unknown LUT kind %d", kind);
  if (dims) std::memcpy(dims, h->dims[kind], sizeof(int32_t) * 3);
  if (device_ptr) *device_ptr = h->lut[kind];
  return ATM_OK;
}

ATM_API int atm_read_lut(const AtmHandle* h, int32_t kind, float* dst_device, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (kind < 0 || kind > 3) return fail(ATM_E_INVALID, "unknown LUT kind %d", kind);
  if (dst_device == nullptr) return fail(ATM_E_INVALID, "null destination");
  ATM_CUDA(atm::launch_lut_to_fields(h->lut[kind], h->dims[kind][0], h->dims[kind][1], h->dims[kind][2], dst_device,
                                     static_cast<cudaStream_t>(stream)),
           "LUT read");
  return ATM_OK;
}

ATM_API int atm_load_lut(AtmHandle* h, int32_t kind, const float* src_device, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (kind < 0 || kind > 3) return fail(ATM_E_INVALID, "unknown LUT kind %d", kind);
  if (src_device == nullptr) return fail(ATM_E_INVALID, "null source");
  ATM_CUDA(atm::launch_fields_to_lut(src_device, h->dims[kind][0], h->dims[kind][1], h->dims[kind][2], h->lut[kind],
                                     static_cast<cudaStream_t>(stream)),
           "LUT load");
  return ATM_OK;
}

ATM_API int atm_read_sample_counter(AtmHandle* h, int32_t reset, uint64_t* out, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long v = 0;
  ATM_CUDA(cudaMemcpyAsync(&v, h->samples, sizeof(v), cudaMemcpyDeviceToHost, s), "sample counter read");
  if (reset) ATM_CUDA(cudaMemsetAsync(h->samples, 0, sizeof(v), s), "sample counter reset");
  ATM_CUDA(cudaStreamSynchronize(s), "sample counter sync");
  if (out) *out = v;
  return ATM_OK;
}

ATM_API int atm_check(AtmHandle* h, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ATM_CUDA(cudaStreamSynchronize(s), "check");
  if (!h->queue) return ATM_OK;
  uint32_t status = 0;
  ATM_CUDA(cudaMemcpy(&status, h->queue + 2, sizeof(status), cudaMemcpyDeviceToHost), "check");
  if (status == 0) return ATM_OK;
  ATM_CUDA(cudaMemset(h->queue + 2, 0, sizeof(status)), "check");
  return fail(ATM_E_TIMEOUT,
              "a tensor-core MMA of atm_composite_surrogate did not complete within its wait bound; the "
              "affected pixels took the plain integrator");
}

// ---- batched builds ------------------------------------------------------
struct AtmBatch {
  std::vector<AtmParams> params;
  std::vector<atm::DevParams> dev;
  std::vector<double> radius;
  std::vector<float4*> tlut, mslut;
  double E[3] = {0, 0, 0};
  double ar_rad = 0.0;
  unsigned char* d_jobs = nullptr;
  size_t jobs_bytes = 0;
  long long* d_prefix = nullptr;
  size_t prefix_count = 0;
  unsigned long long* d_ticket = nullptr;
  unsigned long long* d_samples = nullptr;
  std::vector<unsigned char> h_jobs;
  std::vector<long long> h_prefix;
  int sm_count = 0;
  atm::SurrogateSetDev* d_sets = nullptr;  // surrogate sample generation
};

ATM_API int atm_batch_destroy(AtmBatch* b) {
  if (b == nullptr) return ATM_OK;
  for (float4* p : b->tlut) if (p) cudaFree(p);
  for (float4* p : b->mslut) if (p) cudaFree(p);
  if (b->d_jobs) cudaFree(b->d_jobs);
  if (b->d_prefix) cudaFree(b->d_prefix);
  if (b->d_ticket) cudaFree(b->d_ticket);
  if (b->d_samples) cudaFree(b->d_samples);
  if (b->d_sets) cudaFree(b->d_sets);
  delete b;
  return ATM_OK;
}

ATM_API int atm_batch_create(const AtmParams* sets, const double* planet_radius_m, int32_t n_sets,
                             const double solar_irradiance[3], double sun_angular_radius_degrees, AtmBatch** out,
                             void* stream) {
  if (!sets || !planet_radius_m || !solar_irradiance || !out || n_sets < 1 || n_sets > 1024)
    return fail(ATM_E_INVALID, "atm_batch_create needs 1..1024 parameter sets, radii, irradiance and an output");
  *out = nullptr;
  if (!finite_nonneg3(solar_irradiance) || !std::isfinite(sun_angular_radius_degrees))
    return fail(ATM_E_INVALID, "invalid irradiance or sun angular radius");
  for (int i = 0; i < n_sets; ++i) {
    int rc = validate(sets[i]);
    if (rc) return rc;
    if (!std::isfinite(planet_radius_m[i]) || planet_radius_m[i] <= 1.0)
      return fail(ATM_E_INVALID, "planet radius of set %d must be > 1 m", i);
  }
  AtmBatch* b = new (std::nothrow) AtmBatch();
  if (!b) return fail(ATM_E_NOMEM, "host allocation failed");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::memcpy(b->E, solar_irradiance, sizeof(b->E));
  b->ar_rad = double(radians_f32(sun_angular_radius_degrees));
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ticket, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_samples, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_samples, 0, sizeof(unsigned long long), s);
  for (int i = 0; i < n_sets && e == cudaSuccess; ++i) {
    b->params.push_back(sets[i]);
    b->dev.push_back(atm::make_dev_params(sets[i]));
    b->radius.push_back(planet_radius_m[i]);
    float4 *t = nullptr, *m = nullptr;
    e = cudaMalloc(&t, sizeof(float4) * sets[i].transmittance_lut_width * sets[i].transmittance_lut_height);
    if (e == cudaSuccess)
      e = cudaMalloc(&m, sizeof(float4) * sets[i].multi_scattering_lut_width * sets[i].multi_scattering_lut_height);
    b->tlut.push_back(t);
    b->mslut.push_back(m);
    if (e != cudaSuccess) break;
    float ef[3];
    to_f32(solar_irradiance, ef, 3);
    e = atm::launch_transmittance(b->dev[i], float(planet_radius_m[i]), t, s);
    if (e == cudaSuccess)
      e = atm::launch_multi_scattering(b->dev[i], float(planet_radius_m[i]), ef, float(b->ar_rad), t, m, b->d_samples,
                                       s);
  }
  if (e != cudaSuccess) {
    atm_batch_destroy(b);
    return cuda_fail(e, "batch set-up");
  }
  *out = b;
  return ATM_OK;
}

ATM_API int atm_batch_build(AtmBatch* b, const AtmBatchJob* jobs, int32_t n_jobs, void* arena, int64_t arena_texels,
                            const AtmBatchTuning* tuning, void* stream) {
  if (!b || !jobs || !arena || !tuning || n_jobs < 1) return fail(ATM_E_INVALID, "null argument to atm_batch_build");
  const int sv_item = tuning->sky_view_texels_per_item, ap_item = tuning->aerial_columns_per_item;
  if (sv_item < 1 || sv_item > 4096 || ap_item < 1 || ap_item > 4096 || tuning->blocks_per_sm < 1 ||
      tuning->blocks_per_sm > 8)
    return fail(ATM_E_INVALID, "tuning out of range");
  const size_t jsz = atm::batch_job_size();
  b->h_jobs.assign(size_t(n_jobs) * jsz, 0);
  b->h_prefix.assign(size_t(n_jobs) + 1, 0);
  float4* base = static_cast<float4*>(arena);
  // Processing order: the sky-view jobs, then the aerial volumes (each job
  // writes only its own output range, so the order changes no result).
  // Neighbouring work tickets then run the same LUT kind's warp functions,
  // which keeps the persistent kernel's hot code in the instruction cache.
  std::vector<int> order(static_cast<size_t>(n_jobs));
  for (int i = 0; i < n_jobs; ++i) order[size_t(i)] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return (jobs[a].kind == ATM_LUT_AERIAL) < (jobs[c].kind == ATM_LUT_AERIAL);
  });
  for (int slot = 0; slot < n_jobs; ++slot) {
    const int i = order[size_t(slot)];
    const AtmBatchJob& j = jobs[i];
    if (j.param_set < 0 || j.param_set >= int(b->params.size()))
      return fail(ATM_E_INVALID, "job %d: parameter set %d out of range", i, j.param_set);
    long long texels = 0;
    int units = 0, per = 0;
    if (j.kind == ATM_LUT_SKY_VIEW) {
      if (j.width < 16 || j.width > 2048 || j.height < 16 || j.height > 2048)
        return fail(ATM_E_INVALID, "job %d: sky-view size %dx%d outside 16..2048", i, j.width, j.height);
      texels = (long long)j.width * j.height;
      units = j.width * j.height;
      per = sv_item;
    } else if (j.kind == ATM_LUT_AERIAL) {
      if (j.width < 4 || j.width > 256 || j.height < 4 || j.height > 256 || j.depth < 8 || j.depth > 256)
        return fail(ATM_E_INVALID, "job %d: aerial size %dx%dx%d outside 4..256 x 4..256 x 8..256", i, j.width,
                    j.height, j.depth);
      if (j.frame_width < 1 || j.frame_height < 1 || !(j.tangent_half_fov > 0.0) ||
          !finite_n(j.view_basis, 9) || !finite_n(j.sun_local, 3))
        return fail(ATM_E_INVALID, "job %d: invalid aerial camera", i);
      texels = (long long)j.width * j.height * j.depth;
      units = j.width * j.height;
      per = ap_item;
    } else {
      return fail(ATM_E_INVALID, "job %d: kind %d is not sky-view or aerial", i, j.kind);
    }
    if (j.output_offset < 0 || j.output_offset + texels > arena_texels)
      return fail(ATM_E_INVALID, "job %d: output [%lld, %lld) outside the arena of %lld texels", i,
                  (long long)j.output_offset, (long long)(j.output_offset + texels), (long long)arena_texels);
    if (!std::isfinite(j.camera_altitude_m) || !std::isfinite(j.sun_zenith_cosine))
      return fail(ATM_E_INVALID, "job %d: non-finite camera or sun", i);
    const int p = j.param_set;
    atm::fill_batch_job(*reinterpret_cast<atm::BatchJobDev*>(b->h_jobs.data() + size_t(slot) * jsz), b->dev[p], j,
                        base, b->tlut[p], b->mslut[p], b->radius[p], b->E, b->ar_rad, per);
    b->h_prefix[slot + 1] = b->h_prefix[slot] + (units + per - 1) / per;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (b->jobs_bytes < b->h_jobs.size()) {
    if (b->d_jobs) cudaFree(b->d_jobs);
    b->d_jobs = nullptr;
    b->jobs_bytes = 0;
    ATM_CUDA(cudaMalloc(&b->d_jobs, b->h_jobs.size()), "batch job table");
    b->jobs_bytes = b->h_jobs.size();
  }
  if (b->prefix_count < b->h_prefix.size()) {
    if (b->d_prefix) cudaFree(b->d_prefix);
    b->d_prefix = nullptr;
    b->prefix_count = 0;
    ATM_CUDA(cudaMalloc(&b->d_prefix, b->h_prefix.size() * sizeof(long long)), "batch item prefix");
    b->prefix_count = b->h_prefix.size();
  }
  ATM_CUDA(cudaMemcpyAsync(b->d_jobs, b->h_jobs.data(), b->h_jobs.size(), cudaMemcpyHostToDevice, s), "job upload");
  ATM_CUDA(cudaMemcpyAsync(b->d_prefix, b->h_prefix.data(), b->h_prefix.size() * sizeof(long long),
                           cudaMemcpyHostToDevice, s),
           "prefix upload");
  // the host tables are re-filled by the next call: make sure this one's copies are done
  ATM_CUDA(cudaStreamSynchronize(s), "job upload sync");
  ATM_CUDA(atm::launch_batch(reinterpret_cast<const atm::BatchJobDev*>(b->d_jobs), b->d_prefix, n_jobs,
                             b->h_prefix[n_jobs], b->d_ticket, b->d_samples, b->sm_count * tuning->blocks_per_sm, s),
           "batch launch");
  return ATM_OK;
}

ATM_API int atm_batch_read_samples(AtmBatch* b, int32_t reset, uint64_t* out, void* stream) {
  if (!b) return fail(ATM_E_INVALID, "null AtmBatch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long v = 0;
  ATM_CUDA(cudaMemcpyAsync(&v, b->d_samples, sizeof(v), cudaMemcpyDeviceToHost, s), "batch samples read");
  if (reset) ATM_CUDA(cudaMemsetAsync(b->d_samples, 0, sizeof(v), s), "batch samples reset");
  ATM_CUDA(cudaStreamSynchronize(s), "batch samples sync");
  if (out) *out = v;
  return ATM_OK;
}

ATM_API int atm_batch_static_lut(const AtmBatch* b, int32_t param_set, int32_t kind, void** device_ptr) {
  if (!b || !device_ptr) return fail(ATM_E_INVALID, "null argument");
  if (param_set < 0 || param_set >= int(b->params.size())) return fail(ATM_E_INVALID, "set out of range");
  if (kind == ATM_LUT_TRANSMITTANCE) *device_ptr = b->tlut[param_set];
  else if (kind == ATM_LUT_MULTI_SCATTERING) *device_ptr = b->mslut[param_set];
  else return fail(ATM_E_INVALID, "kind must be transmittance (0) or multi-scattering (1)");
  return ATM_OK;
}

// ---- MLP surrogates -------------------------------------------------------
struct AtmMlp {
  atm::MlpShape shape{};
  float* params = nullptr;
  float* grad = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  float* partial = nullptr;
  size_t partial_floats = 0;
  float* loss_partial = nullptr;
  size_t loss_floats = 0;
  void* packed = nullptr;
  void* packed_tc = nullptr;    // tcgen05 layout (atm_mlp_tc.cuh)
  int* d_error = nullptr;       // set by a tcgen05 kernel whose MMA timed out
  bool packed_current = false;  // packed / packed_tc hold the current parameters
  long long step = 0;
  int sm_count = 0;
};

ATM_API int atm_mlp_destroy(AtmMlp* m) {
  if (!m) return ATM_OK;
  for (void* p : {static_cast<void*>(m->params), static_cast<void*>(m->grad), static_cast<void*>(m->m1),
                  static_cast<void*>(m->m2), static_cast<void*>(m->partial), static_cast<void*>(m->loss_partial),
                  m->packed, m->packed_tc, static_cast<void*>(m->d_error)})
    if (p) cudaFree(p);
  delete m;
  return ATM_OK;
}

ATM_API int atm_mlp_create(int32_t n_in, int32_t n_hidden_layers, int32_t n_out, uint64_t seed, AtmMlp** out) {
  if (!out) return fail(ATM_E_INVALID, "null output");
  *out = nullptr;
  if (n_in < 1 || n_in > 16 || n_out < 1 || n_out > 8 || n_hidden_layers < 1 || n_hidden_layers > 4)
    return fail(ATM_E_INVALID, "MLP shape must have 1..16 inputs, 1..8 outputs and 1..4 hidden layers of 64");
  AtmMlp* m = new (std::nothrow) AtmMlp();
  if (!m) return fail(ATM_E_NOMEM, "host allocation failed");
  m->shape = atm::make_mlp_shape(n_in, n_hidden_layers, n_out);
  const size_t np = size_t(m->shape.n_params);
  // Glorot-uniform weights from a seeded xorshift generator, zero biases
  std::vector<float> host(np, 0.0f);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  auto next = [&st]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return double(st >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < m->shape.n_layers; ++l) {
    const int in = m->shape.in_dim[l], o = m->shape.out_dim[l];
    const double lim = std::sqrt(6.0 / double(in + o));
    for (int i = 0; i < in * o; ++i) host[m->shape.off_w[l] + i] = float((2.0 * next() - 1.0) * lim);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, dev);
  for (float** p : {&m->params, &m->grad, &m->m1, &m->m2})
    if (e == cudaSuccess) e = cudaMalloc(p, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->packed, atm::mlp_bf16_bytes(m->shape));
  if (e == cudaSuccess) e = cudaMalloc(&m->packed_tc, atm::mlp_tc_bytes(m->shape));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_error, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->d_error, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(m->params, host.data(), np * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->m1, 0, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(m->m2, 0, np * sizeof(float));
  if (e != cudaSuccess) {
    atm_mlp_destroy(m);
    return cuda_fail(e, "MLP allocation");
  }
  *out = m;
  return ATM_OK;
}

ATM_API int atm_mlp_info(const AtmMlp* m, int32_t* n_params, float** device_params) {
  if (!m) return fail(ATM_E_INVALID, "null AtmMlp");
  if (n_params) *n_params = m->shape.n_params;
  if (device_params) *device_params = m->params;
  return ATM_OK;
}

ATM_API int atm_mlp_get_params(const AtmMlp* m, float* dst_device, void* stream) {
  if (!m || !dst_device) return fail(ATM_E_INVALID, "null argument");
  ATM_CUDA(cudaMemcpyAsync(dst_device, m->params, size_t(m->shape.n_params) * sizeof(float), cudaMemcpyDeviceToDevice,
                           static_cast<cudaStream_t>(stream)),
           "parameter read");
  return ATM_OK;
}

ATM_API int atm_mlp_set_params(AtmMlp* m, const float* src_device, void* stream) {
  if (!m || !src_device) return fail(ATM_E_INVALID, "null argument");
  ATM_CUDA(cudaMemcpyAsync(m->params, src_device, size_t(m->shape.n_params) * sizeof(float), cudaMemcpyDeviceToDevice,
                           static_cast<cudaStream_t>(stream)),
           "parameter write");
  m->packed_current = false;
  return ATM_OK;
}

ATM_API int atm_mlp_reset_optimizer(AtmMlp* m, void* stream) {
  if (!m) return fail(ATM_E_INVALID, "null AtmMlp");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ATM_CUDA(cudaMemsetAsync(m->m1, 0, size_t(m->shape.n_params) * sizeof(float), s), "optimizer reset");
  ATM_CUDA(cudaMemsetAsync(m->m2, 0, size_t(m->shape.n_params) * sizeof(float), s), "optimizer reset");
  m->step = 0;
  return ATM_OK;
}

namespace {
int mlp_gradient(AtmMlp* m, const float* inputs, const float* targets, const float* weights, int64_t n,
                 float* loss_out, cudaStream_t s) {
  if (!m || !inputs || !targets || n < 1) return fail(ATM_E_INVALID, "invalid MLP gradient arguments");
  const size_t ctas = size_t(atm::mlp_train_ctas(n));
  const size_t need = ctas * size_t(m->shape.n_params);
  if (m->partial_floats < need) {
    if (m->partial) cudaFree(m->partial);
    m->partial = nullptr;
    m->partial_floats = 0;
    ATM_CUDA(cudaMalloc(&m->partial, need * sizeof(float)), "gradient workspace");
    m->partial_floats = need;
  }
  if (m->loss_floats < ctas) {
    if (m->loss_partial) cudaFree(m->loss_partial);
    m->loss_partial = nullptr;
    m->loss_floats = 0;
    ATM_CUDA(cudaMalloc(&m->loss_partial, ctas * sizeof(float)), "loss workspace");
    m->loss_floats = ctas;
  }
  ATM_CUDA(atm::launch_mlp_grad(m->shape, m->params, inputs, targets, weights, n, m->partial, m->loss_partial,
                                m->grad, s),
           "MLP forward/backward");
  if (loss_out) {
    ATM_CUDA(atm::launch_reduce_partials(m->loss_partial, int(ctas), 1, loss_out, s), "loss reduction");
  }
  return ATM_OK;
}
}  // namespace

ATM_API int atm_mlp_gradient(AtmMlp* m, const float* inputs, const float* targets, const float* weights, int64_t n,
                             float* grad_out, float* loss_out, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = mlp_gradient(m, inputs, targets, weights, n, loss_out, s);
  if (rc) return rc;
  if (grad_out)
    ATM_CUDA(cudaMemcpyAsync(grad_out, m->grad, size_t(m->shape.n_params) * sizeof(float), cudaMemcpyDeviceToDevice,
                             s),
             "gradient copy");
  return ATM_OK;
}

ATM_API int atm_mlp_train_step(AtmMlp* m, const float* inputs, const float* targets, const float* weights, int64_t n,
                               float lr, float beta1, float beta2, float eps, float* loss_out, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!(lr > 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) || !(beta2 >= 0.0f && beta2 < 1.0f) || !(eps > 0.0f))
    return fail(ATM_E_INVALID, "invalid Adam hyper-parameters");
  int rc = mlp_gradient(m, inputs, targets, weights, n, loss_out, s);
  if (rc) return rc;
  m->step += 1;
  m->packed_current = false;
  ATM_CUDA(atm::launch_adam(m->params, m->grad, m->m1, m->m2, m->shape.n_params, lr, beta1, beta2, eps, m->step, s),
           "Adam update");
  return ATM_OK;
}

ATM_API int atm_mlp_pack_bf16(AtmMlp* m, void* stream) {
  if (!m) return fail(ATM_E_INVALID, "null AtmMlp");
  ATM_CUDA(atm::launch_mlp_pack_bf16(m->shape, m->params, m->packed, static_cast<cudaStream_t>(stream)),
           "BF16 packing");
  ATM_CUDA(atm::launch_mlp_pack_tc(m->shape, m->params, m->packed_tc, static_cast<cudaStream_t>(stream)),
           "BF16 packing (tcgen05 layout)");
  m->packed_current = true;
  return ATM_OK;
}

ATM_API int atm_mlp_forward(const AtmMlp* m, const float* inputs, float* outputs, int64_t n, int32_t precision,
                            void* stream) {
  if (!m || !inputs || !outputs || n < 1) return fail(ATM_E_INVALID, "invalid MLP forward arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == 0)
    ATM_CUDA(atm::launch_mlp_forward_f32(m->shape, m->params, inputs, outputs, n, s), "MLP forward (FP32)");
  else if (precision == 1)
    ATM_CUDA(atm::launch_mlp_forward_bf16(m->shape, m->packed, inputs, outputs, n, m->sm_count, s),
             "MLP forward (BF16 tensor cores)");
  else if (precision == 2) {
    if (!m->packed_current) return fail(ATM_E_STATE, "network not packed (atm_mlp_pack_bf16)");
    ATM_CUDA(cudaMemsetAsync(m->d_error, 0, sizeof(int), s), "MLP forward (tcgen05)");
    ATM_CUDA(atm::launch_mlp_forward_tc(m->shape, m->packed_tc, inputs, outputs, n, m->d_error, m->sm_count, s),
             "MLP forward (tcgen05)");
    int err = 0;
    ATM_CUDA(cudaMemcpyAsync(&err, m->d_error, sizeof(int), cudaMemcpyDeviceToHost, s), "MLP forward (tcgen05)");
    ATM_CUDA(cudaStreamSynchronize(s), "MLP forward (tcgen05)");
    if (err) return fail(ATM_E_TIMEOUT, "tcgen05 MMA did not complete in time");
  } else
    return fail(ATM_E_INVALID, "precision must be 0 (FP32), 1 (BF16 mma.sync) or 2 (BF16 tcgen05)");
  return ATM_OK;
}

// ---- learned surrogates ----------------------------------------------------
namespace {
bool valid_range(const double* r) {
  return r && std::isfinite(r[0]) && std::isfinite(r[1]) && std::isfinite(r[2]) && std::isfinite(r[3]) &&
         r[0] > 0.0 && r[1] > r[0] && r[2] > 0.0 && r[3] > r[2];
}
// Feature 4 or 5 of a scale height: 2 (ln H - ln lo) / (ln hi - ln lo) - 1.
float log_feature(double H, double lo, double hi) {
  return float(2.0 * (std::log(H) - std::log(lo)) / (std::log(hi) - std::log(lo)) - 1.0);
}
bool mlp_is(const AtmMlp* m, int n_in, int n_hidden, int n_out) {
  return m->shape.n_in == n_in && m->shape.n_out == n_out && m->shape.n_layers == n_hidden + 1;
}
}  // namespace

ATM_API int atm_surrogate_samples(AtmBatch* b, int32_t kind, int64_t n, uint64_t seed,
                                  const AtmSampleOptions* options, const double scale_height_range[4], float* features,
                                  float* targets, void* stream) {
  if (!b || !features || !targets || n < 1) return fail(ATM_E_INVALID, "invalid surrogate sample arguments");
  if (kind != ATM_SURROGATE_SKY && kind != ATM_SURROGATE_AERIAL) return fail(ATM_E_INVALID, "unknown kind %d", kind);
  if (!valid_range(scale_height_range)) return fail(ATM_E_INVALID, "scale-height range must be 0 < min < max");
  atm::SampleShaping shaping{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  if (options) {
    const AtmSampleOptions& o = *options;
    if (!(o.shell_top_fraction >= 0.0 && o.shell_top_fraction <= 1.0 && o.surface_fraction >= 0.0 &&
          o.surface_fraction <= 1.0 && std::isfinite(o.surface_min_m) && std::isfinite(o.surface_max_m) &&
          o.surface_min_m <= o.surface_max_m && std::isfinite(o.start_min_m) && std::isfinite(o.start_max_m) &&
          o.sun_angle_fraction >= 0.0 && o.sun_angle_fraction <= 1.0 && o.sun_angle_max_degrees >= 0.0 &&
          o.sun_angle_max_degrees <= 180.0))
      return fail(ATM_E_INVALID, "sample options out of range");
    shaping = {float(o.shell_top_fraction), float(o.surface_fraction), float(o.surface_min_m),
               float(o.surface_max_m), 0.0f, 0.0f, float(o.sun_angle_fraction),
               float(o.sun_angle_max_degrees * (kPi / 180.0))};
    if (o.start_min_m < o.start_max_m) {
      // the altitude feature 2 sqrt(h / top) - 1 of both ends of the band
      const double top = b->params[0].top_altitude_m;
      if (!(o.start_min_m >= 0.0 && o.start_max_m <= top))
        return fail(ATM_E_INVALID, "start altitude band must lie inside the shell [0, %g] m", top);
      shaping.x0_lo = float(2.0 * std::sqrt(o.start_min_m / top) - 1.0);
      shaping.x0_hi = float(2.0 * std::sqrt(o.start_max_m / top) - 1.0);
    }
  }
  const int n_sets = int(b->params.size());
  for (int i = 1; i < n_sets; ++i)
    if (b->radius[i] != b->radius[0] || b->params[i].top_altitude_m != b->params[0].top_altitude_m)
      return fail(ATM_E_INVALID, "surrogate sample sets must share planet radius and shell top");
  std::vector<atm::SurrogateSetDev> sets(n_sets);
  for (int i = 0; i < n_sets; ++i) {
    const AtmParams& p = b->params[i];
    const double* r = scale_height_range;
    if (p.rayleigh_scale_height_m < r[0] || p.rayleigh_scale_height_m > r[1] || p.mie_scale_height_m < r[2] ||
        p.mie_scale_height_m > r[3])
      return fail(ATM_E_INVALID, "set %d has scale heights outside the feature range", i);
    sets[i].P = b->dev[i];
    sets[i].tlut = b->tlut[i];
    sets[i].mslut = b->mslut[i];
    sets[i].bottom = float(b->radius[i]);
    sets[i].lhr_n = log_feature(p.rayleigh_scale_height_m, r[0], r[1]);
    sets[i].lhm_n = log_feature(p.mie_scale_height_m, r[2], r[3]);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!b->d_sets) ATM_CUDA(cudaMalloc(&b->d_sets, sizeof(atm::SurrogateSetDev) * 1024), "sample set table");
  ATM_CUDA(cudaMemcpyAsync(b->d_sets, sets.data(), sizeof(atm::SurrogateSetDev) * n_sets, cudaMemcpyHostToDevice, s),
           "sample set upload");
  float ef[3];
  to_f32(b->E, ef, 3);
  ATM_CUDA(atm::launch_gen_samples(b->d_sets, n_sets, kind, n, seed, shaping, ef, float(b->ar_rad), features,
                                   targets, b->d_samples, s),
           "surrogate samples");
  // the table is read by the launch: keep the host copy alive until it ran
  ATM_CUDA(cudaStreamSynchronize(s), "surrogate samples");
  return ATM_OK;
}

// Validation of an AtmSurrogate against the frame, and the device-side view
// of its networks, gates and the handle's fallback queue (allocated on first
// use).  Shared by the surrogate composite and the fused frame.
int calibration_setup(AtmHandle* h, const AtmSurrogate* sg, atm::SurrogateQueue& Q, bool sky_pixels = false);
int surrogate_setup(AtmHandle* h, const AtmSurrogate* sg, double planet_radius_m, double camera_radius_m,
                    atm::SurrogateNets& nets, atm::SurrogateQueue& Q) {
  if (!valid_range(sg->scale_height_range)) return fail(ATM_E_INVALID, "scale-height range must be 0 < min < max");
  if (!(sg->check_fraction >= 0.0 && sg->check_fraction <= 1.0))
    return fail(ATM_E_INVALID, "check_fraction must be in [0, 1]");
  if (!(sg->aerial_floor > 0.0 && sg->aerial_floor < 1.0 && sg->sky_floor > 0.0 && sg->sky_floor < 1.0 &&
        sg->aerial_floor_t >= 0.0 && sg->aerial_floor_t < 1.0))
    return fail(ATM_E_INVALID, "radiance floors must be in (0, 1)");
  if (sg->aerial || sg->sky || sg->aerial_above_shell) {
    if (std::fabs(sg->trained_planet_radius_m - planet_radius_m) > 1.0 ||
        std::fabs(sg->trained_top_altitude_m - h->params.top_altitude_m) > 1.0)
      return fail(ATM_E_INVALID, "the networks were trained for another planet radius or shell top");
  }
  nets = atm::SurrogateNets{};
  // the camera above the shell: every segment starts at the shell top
  const bool above = camera_radius_m - planet_radius_m > h->params.top_altitude_m;
  const AtmMlp* aerial = above && sg->aerial_above_shell ? sg->aerial_above_shell : sg->aerial;
  if (aerial) {
    if (!mlp_is(aerial, atm::kSurrogateApIn, atm::kSurrogateApHidden, atm::kSurrogateApOut))
      return fail(ATM_E_INVALID, "aerial network must be 11 -> 4 x 64 -> 6");
    if (!aerial->packed_current) return fail(ATM_E_STATE, "aerial network not packed (atm_mlp_pack_bf16)");
    nets.ap = static_cast<const unsigned char*>(aerial->packed_tc);
    nets.ap_bytes = int(atm::mlp_tc_bytes(aerial->shape));
  }
  if (sg->sky) {
    if (!mlp_is(sg->sky, atm::kSurrogateSkyIn, atm::kSurrogateSkyHidden, atm::kSurrogateSkyOut))
      return fail(ATM_E_INVALID, "sky network must be 10 -> 3 x 64 -> 3");
    if (!sg->sky->packed_current) return fail(ATM_E_STATE, "sky network not packed (atm_mlp_pack_bf16)");
    nets.sky = static_cast<const unsigned char*>(sg->sky->packed_tc);
    nets.sky_bytes = int(atm::mlp_tc_bytes(sg->sky->shape));
  }
  if (nets.ap_bytes % 16 || nets.sky_bytes % 16) return fail(ATM_E_STATE, "packed network size not a multiple of 16");
  const double* r = sg->scale_height_range;
  nets.lhr_n = log_feature(h->params.rayleigh_scale_height_m, r[0], r[1]);
  nets.lhm_n = log_feature(h->params.mie_scale_height_m, r[2], r[3]);
  if (!(sg->twilight_cosine >= 0.0 && sg->twilight_cosine <= 1.0 && sg->sky_twilight_cosine >= 0.0 &&
        sg->sky_twilight_cosine <= 1.0 && sg->limb_degrees >= 0.0 && sg->limb_degrees <= 90.0))
    return fail(ATM_E_INVALID, "gate thresholds out of range");
  nets.twilight_cos = float(sg->twilight_cosine);
  nets.sky_twilight_cos = float(sg->sky_twilight_cosine);
  nets.limb_rad = float(sg->limb_degrees * (kPi / 180.0));
  nets.floor = float(sg->aerial_floor);
  nets.floor_t = float(sg->aerial_floor_t);
  nets.sky_floor = float(sg->sky_floor);
  if (sg->tc_wait_polls < -1) return fail(ATM_E_INVALID, "tc_wait_polls must be -1, 0 or positive");
  nets.wait_tries = sg->tc_wait_polls == 0 ? atm::kTcWaitTries : sg->tc_wait_polls < 0 ? 0 : sg->tc_wait_polls;
  nets.gate_crossing = sg->gate_terminator != 0;
  if (!h->queue) {
    const size_t cap = size_t(h->width) * size_t(h->height);
    ATM_CUDA(cudaMalloc(&h->queue, (cap + 4) * sizeof(uint32_t)), "fallback queue");
    ATM_CUDA(cudaMemset(h->queue, 0, 4 * sizeof(uint32_t)), "fallback queue");
    int dev = 0;
    ATM_CUDA(cudaGetDevice(&dev), "device query");
    ATM_CUDA(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, dev), "device query");
  }
  Q = atm::SurrogateQueue{};
  Q.count = h->queue;
  Q.status = h->queue + 2;
  Q.items = h->queue + 4;
  Q.stats = sg->stats;
  Q.check_fraction = float(sg->check_fraction);
  if (int rc = calibration_setup(h, sg, Q)) return rc;
  Q.seed = sg->seed;
  return ATM_OK;
}

// The checked pixels' calibration (AtmSurrogate.calibration_tile): the
// handle's scratch image and tile sums (allocated on first use) into Q.
int calibration_setup(AtmHandle* h, const AtmSurrogate* sg, atm::SurrogateQueue& Q, bool sky_pixels) {
  if (sg->calibration_tile == 0) return ATM_OK;
  const int t = sg->calibration_tile;
  if (t < 16 || t > 256 || (t & (t - 1)) != 0)
    return fail(ATM_E_INVALID, "calibration_tile must be 0 or a power of two in 16..256");
  if (!h->calib_tiles) {
    const size_t tiles = size_t((h->width + 15) / 16) * size_t((h->height + 15) / 16);
    ATM_CUDA(cudaMalloc(&h->calib_tiles, tiles * 4 * sizeof(float)), "calibration tiles");
  }
  Q.tiles = h->calib_tiles;
  Q.tile_shift = 0;
  while ((1 << Q.tile_shift) < t) ++Q.tile_shift;
  Q.tiles_x = (h->width + t - 1) / t;
  if (sky_pixels) {  // the output holds the network radiance: a byte mask suffices
    if (!h->calib_mask)
      ATM_CUDA(cudaMalloc(&h->calib_mask, size_t(h->width) * size_t(h->height)), "calibration mask");
    Q.net_mask = h->calib_mask;
    return ATM_OK;
  }
  if (!h->calib_lm) {
    const size_t px = size_t(h->width) * size_t(h->height);
    ATM_CUDA(cudaMalloc(&h->calib_lm, px * 3 * sizeof(float)), "calibration scratch");
  }
  Q.lm = h->calib_lm;
  return ATM_OK;
}

ATM_API int atm_composite_surrogate(AtmHandle* h, const float* scene_hdr, const float* space_hdr,
                                    const int32_t* surface_id, const float* position_view, float* hdr,
                                    const AtmImage* image, double planet_radius_m, double camera_radius_m,
                                    const double sun_local[3], const double solar_irradiance[3],
                                    const double sun_disk_radiance[3], double sun_angular_radius_degrees,
                                    const double view_basis[9], double tangent_half_fov, double star_contrast_start,
                                    double star_contrast_end, const AtmSurrogate* sg, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = check_image(h, image))) return rc;
  if (!scene_hdr || !space_hdr || !surface_id || !position_view || !hdr || !sun_local || !solar_irradiance ||
      !sun_disk_radiance || !view_basis || !sg)
    return fail(ATM_E_INVALID, "null pointer argument to atm_composite_surrogate");
  if (!finite_n(view_basis, 9) || !finite_n(sun_local, 3) || !std::isfinite(tangent_half_fov) ||
      tangent_half_fov <= 0.0)
    return fail(ATM_E_INVALID, "non-finite or non-positive frame argument");
  if (int64_t(image->width) * image->height > (int64_t(1) << 30))
    return fail(ATM_E_INVALID, "frame larger than 2^30 pixels");
  atm::SurrogateNets nets{};
  atm::SurrogateQueue Q{};
  if ((rc = surrogate_setup(h, sg, planet_radius_m, camera_radius_m, nets, Q))) return rc;
  const atm::CompositeScalars A =
      composite_scalars(h, planet_radius_m, camera_radius_m, sun_local, solar_irradiance, sun_disk_radiance,
                        sun_angular_radius_degrees, view_basis, tangent_half_fov, star_contrast_start,
                        star_contrast_end);
  ATM_CUDA(atm::launch_composite_surrogate(h->dev, layout_of(image), A, scene_hdr, space_hdr, surface_id,
                                           position_view, h->lut[ATM_LUT_TRANSMITTANCE],
                                           h->lut[ATM_LUT_MULTI_SCATTERING], h->lut[ATM_LUT_SKY_VIEW], nets, Q, hdr,
                                           h->samples, h->sm_count, static_cast<cudaStream_t>(stream)),
           "surrogate composite");
  return ATM_OK;
}

ATM_API int atm_sky_pixels(AtmHandle* h, int32_t mode, float* radiance, const AtmImage* image,
                           double planet_radius_m, double camera_radius_m, const double sun_local[3],
                           const double solar_irradiance[3], double sun_angular_radius_degrees,
                           const double view_basis[9], double tangent_half_fov, const AtmSurrogate* sg,
                           void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = check_image(h, image))) return rc;
  if (!radiance || !sun_local || !solar_irradiance || !view_basis)
    return fail(ATM_E_INVALID, "null pointer argument to atm_sky_pixels");
  if (mode < ATM_SKY_PIXELS_PLAIN || mode > ATM_SKY_PIXELS_LUT) return fail(ATM_E_INVALID, "unknown mode %d", mode);
  if (!finite_n(view_basis, 9) || !finite_n(sun_local, 3) || !std::isfinite(tangent_half_fov) ||
      tangent_half_fov <= 0.0)
    return fail(ATM_E_INVALID, "non-finite or non-positive frame argument");
  atm::SurrogateNets nets{};
  if (mode == ATM_SKY_PIXELS_NET) {
    if (!sg || !sg->sky) return fail(ATM_E_INVALID, "the network mode needs a surrogate with a sky network");
    if (!mlp_is(sg->sky, atm::kSurrogateSkyIn, atm::kSurrogateSkyHidden, atm::kSurrogateSkyOut))
      return fail(ATM_E_INVALID, "sky network must be 10 -> 3 x 64 -> 3");
    if (!sg->sky->packed_current) return fail(ATM_E_STATE, "sky network not packed (atm_mlp_pack_bf16)");
    if (!valid_range(sg->scale_height_range)) return fail(ATM_E_INVALID, "scale-height range must be 0 < min < max");
    if (std::fabs(sg->trained_planet_radius_m - planet_radius_m) > 1.0 ||
        std::fabs(sg->trained_top_altitude_m - h->params.top_altitude_m) > 1.0)
      return fail(ATM_E_INVALID, "the networks were trained for another planet radius or shell top");
    if (!(sg->sky_floor > 0.0 && sg->sky_floor < 1.0)) return fail(ATM_E_INVALID, "radiance floors must be in (0, 1)");
    if (!(sg->sky_twilight_cosine >= 0.0 && sg->sky_twilight_cosine <= 1.0 && sg->limb_degrees >= 0.0 &&
          sg->limb_degrees <= 90.0))
      return fail(ATM_E_INVALID, "gate thresholds out of range");
    if (sg->tc_wait_polls < -1) return fail(ATM_E_INVALID, "tc_wait_polls must be -1, 0 or positive");
    nets.sky = static_cast<const unsigned char*>(sg->sky->packed_tc);
    nets.sky_bytes = int(atm::mlp_tc_bytes(sg->sky->shape));
    if (nets.sky_bytes % 16) return fail(ATM_E_STATE, "packed network size not a multiple of 16");
    const double* r = sg->scale_height_range;
    nets.lhr_n = log_feature(h->params.rayleigh_scale_height_m, r[0], r[1]);
    nets.lhm_n = log_feature(h->params.mie_scale_height_m, r[2], r[3]);
    nets.sky_floor = float(sg->sky_floor);
    nets.sky_twilight_cos = float(sg->sky_twilight_cosine);
    nets.limb_rad = float(sg->limb_degrees * (kPi / 180.0));
    nets.wait_tries =
        sg->tc_wait_polls == 0 ? atm::kTcWaitTries : sg->tc_wait_polls < 0 ? 0 : sg->tc_wait_polls;
  }
  if (mode == ATM_SKY_PIXELS_LUT && !h->sky_valid)
    return fail(ATM_E_STATE, "the LUT mode needs a sky-view LUT (atm_update first)");
  if (!h->queue) {  // the timeout flag lives in the fallback queue's header
    const size_t cap = size_t(h->width) * size_t(h->height);
    ATM_CUDA(cudaMalloc(&h->queue, (cap + 4) * sizeof(uint32_t)), "fallback queue");
    ATM_CUDA(cudaMemset(h->queue, 0, 4 * sizeof(uint32_t)), "fallback queue");
    int dev = 0;
    ATM_CUDA(cudaGetDevice(&dev), "device query");
    ATM_CUDA(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, dev), "device query");
  }
  const double zero3[3] = {0.0, 0.0, 0.0};
  const atm::CompositeScalars A =
      composite_scalars(h, planet_radius_m, camera_radius_m, sun_local, solar_irradiance, zero3,
                        sun_angular_radius_degrees, view_basis, tangent_half_fov, 0.0, 1.0);
  atm::SurrogateQueue Q{};
  if (mode == ATM_SKY_PIXELS_NET) {  // the checked pixels' calibration of the sky network
    if (!(sg->check_fraction >= 0.0 && sg->check_fraction <= 1.0))
      return fail(ATM_E_INVALID, "check_fraction must be in [0, 1]");
    Q.count = h->queue;
    Q.status = h->queue + 2;
    Q.items = h->queue + 4;
    Q.check_fraction = float(sg->check_fraction);
    Q.seed = sg->seed;
    if (int rc2 = calibration_setup(h, sg, Q, true)) return rc2;
  }
  ATM_CUDA(atm::launch_sky_pixels(mode, h->dev, layout_of(image), A, h->lut[ATM_LUT_TRANSMITTANCE],
                                  h->lut[ATM_LUT_MULTI_SCATTERING], h->lut[ATM_LUT_SKY_VIEW], nets, h->queue + 2,
                                  radiance, h->samples, h->sm_count, static_cast<cudaStream_t>(stream), &Q),
           "sky pixels");
  return ATM_OK;
}

// Composite that allocates nothing (no counterpart in the reference).  See
// include/atm_capi.h: caller-owned LUTs, images and count output; the only
// scratch is the library's file-scope per-tile array.
ATM_API int atm_composite_noalloc(const AtmParams* params, const void* transmittance_lut,
                                  const void* multi_scattering_lut, const void* sky_view_lut,
                                  const float* scene_hdr, const float* space_hdr, const int32_t* surface_id,
                                  const float* position_view, float* hdr, const AtmImage* image,
                                  double planet_radius_m, double camera_radius_m, double sky_lut_camera_altitude_m,
                                  const double sun_local[3], const double solar_irradiance[3],
                                  const double sun_disk_radiance[3], double sun_angular_radius_degrees,
                                  const double view_basis[9], double tangent_half_fov, double star_contrast_start,
                                  double star_contrast_end, uint64_t* samples_out, void* stream) {
  if (params == nullptr) return fail(ATM_E_INVALID, "null AtmParams");
  int rc = validate(*params);
  if (rc) return rc;
  if (!transmittance_lut || !multi_scattering_lut || !sky_view_lut || !scene_hdr || !space_hdr || !surface_id ||
      !position_view || !hdr || !image || !sun_local || !solar_irradiance || !sun_disk_radiance || !view_basis)
    return fail(ATM_E_INVALID, "null pointer argument to atm_composite_noalloc");
  if (image->width < 1 || image->height < 1 || image->stride_x <= 0 || image->stride_y <= 0 ||
      (image->channels != 3 && image->channels != 4))
    return fail(ATM_E_INVALID, "invalid AtmImage");
  if (image->width > 16384 || image->height > 16384)
    return fail(ATM_E_INVALID, "frame %dx%d: width and height are limited to 16384, as for atm_create",
                image->width, image->height);
  const long long tiles = (long long)((image->width + 15) / 16) * ((image->height + 15) / 16);
  if (tiles > atm::noalloc_max_tiles())
    return fail(ATM_E_INVALID,
                "frame %dx%d needs %lld 16x16 tiles; atm_composite_noalloc's fixed scratch holds %d tiles "
                "(16.7 million pixels): use atm_composite for larger frames",
                image->width, image->height, tiles, atm::noalloc_max_tiles());
  if (!finite_n(view_basis, 9) || !finite_n(sun_local, 3) || !std::isfinite(tangent_half_fov) ||
      tangent_half_fov <= 0.0 || !std::isfinite(planet_radius_m) || !std::isfinite(camera_radius_m))
    return fail(ATM_E_INVALID, "non-finite or non-positive frame argument");
  uint32_t* scratch = nullptr;
  ATM_CUDA(atm::noalloc_tile_scratch(&scratch, static_cast<cudaStream_t>(stream)),
           "no-allocation scratch set-up (cudaGetSymbolAddress; make the first call on a device before any capture)");
  const double alt = std::fmax(camera_radius_m - planet_radius_m, 0.0);
  atm::CompositeScalars A{};
  A.bottom = float(planet_radius_m);
  A.cam_alt = float(alt);
  A.sky_alt = float(sky_lut_camera_altitude_m);
  A.ar = radians_f32(sun_angular_radius_degrees);
  A.tanfov = float(tangent_half_fov);
  A.star_start = float(star_contrast_start);
  A.star_end = float(star_contrast_end);
  to_f32(sun_local, A.sun, 3);
  to_f32(solar_irradiance, A.E, 3);
  to_f32(sun_disk_radiance, A.disk, 3);
  to_f32(view_basis, A.right, 3);
  to_f32(view_basis + 3, A.up, 3);
  to_f32(view_basis + 6, A.fwd, 3);
  A.view = ATM_VIEW_COMPOSITE;
  ATM_CUDA(atm::launch_composite_noalloc(atm::make_dev_params(*params), layout_of(image), A, scene_hdr, space_hdr,
                                         surface_id, position_view, static_cast<const float4*>(transmittance_lut),
                                         static_cast<const float4*>(multi_scattering_lut),
                                         static_cast<const float4*>(sky_view_lut), hdr, scratch,
                                         reinterpret_cast<unsigned long long*>(samples_out),
                                         static_cast<cudaStream_t>(stream)),
           "composite (no allocation)");
  return ATM_OK;
}

// ---- display post-process ----------------------------------------------------
struct AtmPost {
  AtmPostConfig config{};
  int32_t width = 0, height = 0;
  atm::PostParams params{};
  float4* bloom_a = nullptr;
  float4* bloom_b = nullptr;
  const float4* last_bloom = nullptr;
  int last_x_fast = 1;  // orientation of last_bloom's storage
};

namespace {

// PostprocessConfig.__post_init__ (postprocess.py:21-38), same messages.
int check_post_config(const AtmPostConfig* c) {
  if (!c) return fail(ATM_E_INVALID, "null AtmPostConfig");
  if (!std::isfinite(c->exposure_ev) || !(c->exposure_ev >= -20.0 && c->exposure_ev <= 20.0))
    return fail(ATM_E_INVALID, "postprocess.exposure_ev must be finite and in [-20, 20]");
  const struct {
    const char* name;
    double value;
  } fields[] = {{"bloom_threshold", c->bloom_threshold},
                {"bloom_knee", c->bloom_knee},
                {"bloom_clamp", c->bloom_clamp},
                {"bloom_strength", c->bloom_strength}};
  for (const auto& f : fields)
    if (!std::isfinite(f.value) || f.value < 0.0)
      return fail(ATM_E_INVALID, "postprocess.%s must be finite and non-negative", f.name);
  if (c->bloom_passes < 0 || c->bloom_passes > 8) return fail(ATM_E_INVALID, "postprocess.bloom_passes must be in 0..8");
  return ATM_OK;
}

}  // namespace

ATM_API int atm_post_destroy(AtmPost* p) {
  if (!p) return ATM_OK;
  if (p->bloom_a) cudaFree(p->bloom_a);
  if (p->bloom_b) cudaFree(p->bloom_b);
  delete p;
  return ATM_OK;
}

ATM_API int atm_post_create(const AtmPostConfig* config, int32_t width, int32_t height, AtmPost** out) {
  if (!out) return fail(ATM_E_INVALID, "null output");
  *out = nullptr;
  int rc;
  if ((rc = check_post_config(config))) return rc;
  if (width < 1 || height < 1) return fail(ATM_E_INVALID, "post-process size must be at least 1x1");
  AtmPost* p = new (std::nothrow) AtmPost();
  if (!p) return fail(ATM_E_NOMEM, "host allocation failed");
  p->config = *config;
  p->width = width;
  p->height = height;
  atm::PostParams& Q = p->params;
  Q.hw = std::max((width + 1) / 2, 1);  // PostProcessor.__init__ :81-82
  Q.hh = std::max((height + 1) / 2, 1);
  Q.threshold = float(config->bloom_threshold);
  Q.knee = float(config->bloom_knee);
  Q.two_knee = float(2.0 * config->bloom_knee);
  Q.knee_div = float(std::max(4.0 * config->bloom_knee, 1.0e-6));
  Q.clamp = float(config->bloom_clamp);
  const size_t bytes = size_t(Q.hw) * size_t(Q.hh) * sizeof(float4);
  cudaError_t e = cudaMalloc(&p->bloom_a, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&p->bloom_b, bytes);
  if (e == cudaSuccess) e = cudaMemset(p->bloom_a, 0, bytes);
  if (e != cudaSuccess) {
    atm_post_destroy(p);
    return cuda_fail(e, "post-process allocation");
  }
  p->last_bloom = p->bloom_a;
  *out = p;
  return ATM_OK;
}

ATM_API int atm_post_process(AtmPost* p, const float* hdr, float* display, const AtmImage* image, double exposure_ev,
                             int32_t bloom, int32_t tone_map, void* stream) {
  if (!p) return fail(ATM_E_INVALID, "null AtmPost");
  if (!hdr || !display) return fail(ATM_E_INVALID, "null image pointer");
  if (!image) return fail(ATM_E_INVALID, "null AtmImage");
  if (image->width != p->width || image->height != p->height)
    return fail(ATM_E_INVALID, "image is %dx%d but the post-process was created for %dx%d", image->width,
                image->height, p->width, p->height);
  if (image->channels != 3 && image->channels != 4) return fail(ATM_E_INVALID, "channels must be 3 or 4");
  if (image->stride_x <= 0 || image->stride_y <= 0) return fail(ATM_E_INVALID, "image strides must be positive");
  // PostProcessor.process :176-207: the multiplier and strength are f32 kernel arguments
  const float exposure = tone_map ? float(std::pow(2.0, exposure_ev)) : 1.0f;
  const bool use_bloom = bloom && p->config.bloom_passes > 0 && p->config.bloom_strength > 0.0;
  const float4* result = nullptr;
  atm::PostParams Q = p->params;
  Q.x_fast = atm::image_x_fast(layout_of(image)) ? 1 : 0;
  ATM_CUDA(atm::launch_post(Q, layout_of(image), hdr, display, p->bloom_a, p->bloom_b, exposure,
                            float(p->config.bloom_strength), p->config.bloom_passes, use_bloom, tone_map != 0,
                            &result, static_cast<cudaStream_t>(stream)),
           "post-process");
  if (use_bloom) {
    p->last_bloom = result;
    p->last_x_fast = Q.x_fast;
  }
  return ATM_OK;
}

ATM_API int atm_post_read_bloom(const AtmPost* p, int32_t dims[2], float* dst_device, void* stream) {
  if (!p) return fail(ATM_E_INVALID, "null AtmPost");
  if (dims) {
    dims[0] = p->params.hw;
    dims[1] = p->params.hh;
  }
  if (dst_device) {
    atm::PostParams Q = p->params;
    Q.x_fast = p->last_x_fast;
    ATM_CUDA(atm::launch_post_read_bloom(Q, p->last_bloom, reinterpret_cast<float4*>(dst_device),
                                         static_cast<cudaStream_t>(stream)),
             "bloom read");
  }
  return ATM_OK;
}

// ---- surface shading -------------------------------------------------------------
// AtmShadeParams in the float32 form of the reference kernel's arguments;
// the images of `im` the shading reads are checked (with_lighting: also the
// surface lighting and the output of a separate shading pass).
int shade_setup(const AtmShadeParams* p, const AtmShadeImages* im, bool with_lighting, atm::ShadeParams& S,
                atm::ShadeImages& I) {
  if (!p || !im) return fail(ATM_E_INVALID, "null shading argument");
  const void* required[] = {im->position,       im->normal,          im->albedo,         im->water_depth,
                            im->seabed_albedo,  im->seabed_normal,   im->slope_variance, im->surface_id,
                            im->terrain_position, im->terrain_normal, im->terrain_albedo, im->terrain_surface_id};
  for (const void* q : required)
    if (!q) return fail(ATM_E_INVALID, "null image pointer");
  if (with_lighting && (!im->sun_transmittance || !im->sky_radiance || !im->surface_hdr))
    return fail(ATM_E_INVALID, "null image pointer");
  const double* finite[] = {p->sun_global, p->solar_irradiance, p->view_right_global, p->view_up_global,
                            p->view_forward_global, p->ocean_absorption, p->ocean_scattering};
  for (const double* v : finite)
    if (!finite_n(v, 3)) return fail(ATM_E_INVALID, "vector arguments must be finite");
  S = atm::ShadeParams{};
  to_f32(p->sun_global, S.sun, 3);
  to_f32(p->solar_irradiance, S.E, 3);
  to_f32(p->view_right_global, S.right, 3);
  to_f32(p->view_up_global, S.up, 3);
  to_f32(p->view_forward_global, S.fwd, 3);
  S.advanced = p->advanced_ocean_enabled != 0;
  S.mode = p->mode;
  S.roughness = float(p->ocean_roughness);
  S.f0 = float(p->ocean_f0);
  S.sky_strength = float(p->ocean_sky_strength);
  for (int k = 0; k < 3; ++k) {  // renderer.py:1521, :1546-1549, in float32
    S.extinction[k] = float(p->ocean_absorption[k]) + float(p->ocean_scattering[k]);
    S.scattering_albedo[k] = float(p->ocean_scattering[k]) / std::max(S.extinction[k], 1.0e-6f);
  }
  S.max_depth = float(p->ocean_max_depth);
  S.eta = 1.0f / float(p->ocean_refraction_index);  // :1402
  S.strength = float(p->ocean_refraction_strength);
  S.max_offset = float(p->ocean_refraction_max_offset_pixels);
  const float t = std::tan(float(p->sun_angular_radius));  // :1345
  S.solar_slope_variance = t * t;
  S.tanfov = float(p->tangent_half_fov);
  S.four_pi = float(4.0 * kPi);
  S.ocean_id = p->ocean_surface_id;
  I = atm::ShadeImages{im->position,       im->normal,         im->albedo,         im->water_depth,
                       im->seabed_albedo,  im->seabed_normal,  im->slope_variance, im->surface_id,
                       im->terrain_position, im->terrain_normal, im->terrain_albedo, im->terrain_surface_id,
                       im->sun_transmittance, im->sky_radiance, im->surface_hdr};
  return ATM_OK;
}

ATM_API int atm_shade_surface(const AtmShadeParams* p, const AtmShadeImages* im, const AtmImage* image,
                              void* stream) {
  if (!p || !im || !image) return fail(ATM_E_INVALID, "null argument");
  if (image->width < 1 || image->height < 1) return fail(ATM_E_INVALID, "image must be at least 1x1");
  if (image->channels != 3 && image->channels != 4) return fail(ATM_E_INVALID, "channels must be 3 or 4");
  if (image->stride_x <= 0 || image->stride_y <= 0) return fail(ATM_E_INVALID, "image strides must be positive");
  atm::ShadeParams S;
  atm::ShadeImages I;
  int rc = shade_setup(p, im, true, S, I);
  if (rc) return rc;
  ATM_CUDA(atm::launch_shade_surface(S, layout_of(image), I, static_cast<cudaStream_t>(stream)), "surface shading");
  return ATM_OK;
}

ATM_API int atm_render_frame(AtmHandle* h, const AtmShadeParams* shade, const AtmShadeImages* images,
                             const float* space_hdr, float* hdr, const AtmImage* image, double planet_radius_m,
                             double camera_radius_m, const double sun_local[3], const double solar_irradiance[3],
                             const double sun_disk_radiance[3], double sun_angular_radius_degrees,
                             const double view_basis[9], double tangent_half_fov, double star_contrast_start,
                             double star_contrast_end, const AtmSurrogate* sg, void* stream) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = check_image(h, image))) return rc;
  if (!space_hdr || !hdr || !sun_local || !solar_irradiance || !sun_disk_radiance || !view_basis)
    return fail(ATM_E_INVALID, "null pointer argument to atm_render_frame");
  if (!finite_n(view_basis, 9) || !finite_n(sun_local, 3) || !std::isfinite(tangent_half_fov) ||
      tangent_half_fov <= 0.0)
    return fail(ATM_E_INVALID, "non-finite or non-positive frame argument");
  atm::ShadeParams S;
  atm::ShadeImages I;
  if ((rc = shade_setup(shade, images, false, S, I))) return rc;
  if (!h->t_valid || !h->ms_valid || !h->sky_valid)
    return fail(ATM_E_STATE, "the frame needs the renderer's LUTs (atm_update first)");
  const atm::CompositeScalars A =
      composite_scalars(h, planet_radius_m, camera_radius_m, sun_local, solar_irradiance, sun_disk_radiance,
                        sun_angular_radius_degrees, view_basis, tangent_half_fov, star_contrast_start,
                        star_contrast_end);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const atm::ImageLayout L = layout_of(image);
  if (sg == nullptr) {
    ATM_CUDA(atm::launch_frame(h->dev, L, A, S, I, space_hdr, h->lut[ATM_LUT_TRANSMITTANCE],
                               h->lut[ATM_LUT_MULTI_SCATTERING], h->lut[ATM_LUT_SKY_VIEW], hdr, h->samples, s),
             "fused frame");
    return ATM_OK;
  }
  atm::SurrogateNets nets{};
  atm::SurrogateQueue Q{};
  if ((rc = surrogate_setup(h, sg, planet_radius_m, camera_radius_m, nets, Q))) return rc;
  ATM_CUDA(atm::launch_composite_surrogate(h->dev, L, A, nullptr, space_hdr, images->surface_id, images->position,
                                           h->lut[ATM_LUT_TRANSMITTANCE], h->lut[ATM_LUT_MULTI_SCATTERING],
                                           h->lut[ATM_LUT_SKY_VIEW], nets, Q, hdr, h->samples, h->sm_count, s, &S, &I),
           "fused surrogate frame");
  return ATM_OK;
}

// ---- terrain raster ----------------------------------------------------------
struct AtmRaster {
  int32_t width = 0, height = 0, max_patches = 0, triangles_per_patch = 0;
  atm::RasterTri* tris = nullptr;
  long long capacity = 0;
  uint32_t* count = nullptr;  // emitted, large, spare
  uint32_t* large = nullptr;
  uint32_t* large_tiles = nullptr;
  unsigned long long* tile_prefix = nullptr;
  unsigned long long* block_sums = nullptr;
  unsigned long long* depth_key = nullptr;
  int sm_count = 0;
};

ATM_API int atm_raster_create(int32_t width, int32_t height, int32_t max_patches, int32_t triangles_per_patch,
                              AtmRaster** out) {
  if (!out) return fail(ATM_E_INVALID, "null output pointer");
  *out = nullptr;
  if (width < 1 || height < 1 || width > 16384 || height > 16384)
    return fail(ATM_E_INVALID, "raster size must be 1..16384 a side");
  if (max_patches < 1 || triangles_per_patch < 1)
    return fail(ATM_E_INVALID, "max_patches and triangles_per_patch must be positive");
  const long long capacity = (long long)max_patches * triangles_per_patch * 6;  // MAX_CLIPPED_TRIANGLES
  if (capacity > 0xffffffffll) return fail(ATM_E_INVALID, "triangle stream over 2^32 triangles");
  AtmRaster* r = new (std::nothrow) AtmRaster;
  if (!r) return fail(ATM_E_NOMEM, "host allocation failed");
  r->width = width;
  r->height = height;
  r->max_patches = max_patches;
  r->triangles_per_patch = triangles_per_patch;
  r->capacity = capacity;
  cudaError_t e = cudaMalloc(&r->tris, sizeof(atm::RasterTri) * size_t(capacity));
  if (e == cudaSuccess) e = cudaMalloc(&r->count, 4 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&r->large, sizeof(uint32_t) * size_t(capacity));
  if (e == cudaSuccess) e = cudaMalloc(&r->large_tiles, sizeof(uint32_t) * size_t(capacity));
  if (e == cudaSuccess) e = cudaMalloc(&r->tile_prefix, sizeof(unsigned long long) * (size_t(capacity) + 1));
  if (e == cudaSuccess) e = cudaMalloc(&r->block_sums, sizeof(unsigned long long) * (atm::kRasterScanBlocks + 1));
  if (e == cudaSuccess) e = cudaMalloc(&r->depth_key, sizeof(unsigned long long) * size_t(width) * height);
  int dev = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&r->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) {
    atm_raster_destroy(r);
    return e == cudaErrorMemoryAllocation ? fail(ATM_E_NOMEM, "raster allocation failed") : cuda_fail(e, "raster");
  }
  *out = r;
  return ATM_OK;
}

ATM_API int atm_raster_destroy(AtmRaster* r) {
  if (!r) return ATM_OK;
  if (r->tris) cudaFree(r->tris);
  if (r->count) cudaFree(r->count);
  if (r->large) cudaFree(r->large);
  if (r->tile_prefix) cudaFree(r->tile_prefix);
  if (r->large_tiles) cudaFree(r->large_tiles);
  if (r->block_sums) cudaFree(r->block_sums);
  if (r->depth_key) cudaFree(r->depth_key);
  delete r;
  return ATM_OK;
}

ATM_API int atm_raster_terrain(AtmRaster* r, const AtmRasterMesh* m, double near_m, double tangent_half_fov,
                               int32_t view_mode, const AtmRasterOutputs* o, const AtmImage* image, void* stream) {
  if (!r || !m || !o || !image) return fail(ATM_E_INVALID, "null argument to atm_raster_terrain");
  if (image->width != r->width || image->height != r->height)
    return fail(ATM_E_INVALID, "image is %dx%d but the raster was created for %dx%d", image->width, image->height,
                r->width, r->height);
  if ((image->channels != 3 && image->channels != 4) || image->stride_x <= 0 || image->stride_y <= 0)
    return fail(ATM_E_INVALID, "invalid AtmImage");
  if (!m->view || !m->normal || !m->material || !m->height_m || !m->cell || !m->triangles ||
      (m->n_active > 0 && !m->active_slots))
    return fail(ATM_E_INVALID, "null mesh array");
  if (!o->depth || !o->position || !o->normal || !o->albedo || !o->material_weights || !o->height_m ||
      !o->surface_id || !o->cell_id)
    return fail(ATM_E_INVALID, "null output image");
  if (m->patches < 1 || m->patches > r->max_patches || m->triangles_per_patch != r->triangles_per_patch ||
      m->vertices_per_patch < 3 || m->n_active < 0 || m->n_active > m->patches ||
      m->surface_triangles_per_patch < 0 || m->surface_triangles_per_patch > m->triangles_per_patch ||
      m->resolution < 1)
    return fail(ATM_E_INVALID, "mesh sizes do not match the raster (patches %d of %d, triangles %d of %d)",
                m->patches, r->max_patches, m->triangles_per_patch, r->triangles_per_patch);
  if (m->triangles_per_patch > m->surface_triangles_per_patch &&
      (m->triangles_per_patch - m->surface_triangles_per_patch) > 8 * m->resolution)
    return fail(ATM_E_INVALID, "at most 4 edges x 2 resolution skirt triangles");
  if (view_mode < 0 || view_mode > 3) return fail(ATM_E_INVALID, "view_mode must be 0..3");
  if (view_mode == 2 && !m->slot_level) return fail(ATM_E_INVALID, "view mode 2 needs slot_level");
  if (!(near_m > 0.0) || !(tangent_half_fov > 0.0) || !std::isfinite(near_m) || !std::isfinite(tangent_half_fov))
    return fail(ATM_E_INVALID, "near plane and field of view must be positive and finite");
  // host-side checks of the topology and active list (small arrays, device
  // resident: validated once by a copy would need a sync; the kernels clamp
  // nothing, so the caller's indices must be in range)
  atm::RasterMeshDev M{m->view,       m->normal,     m->material,  m->height_m,
                       m->cell,       m->triangles,  m->active_slots, m->skirt_mask,
                       m->slot_level, m->patches,    m->vertices_per_patch, m->triangles_per_patch,
                       m->surface_triangles_per_patch, m->resolution, m->n_active};
  atm::RasterStream S{r->tris, r->count, r->capacity, r->large, r->large_tiles, r->tile_prefix, r->block_sums};
  if (o->terrain_surface_id && (!o->terrain_position || !o->terrain_normal || !o->terrain_albedo))
    return fail(ATM_E_INVALID, "the terrain snapshot needs position, normal and albedo images");
  atm::RasterOutDev O{o->depth,          o->position,        o->normal,           o->albedo,
                      o->material_weights, o->height_m,      o->surface_id,       o->cell_id,
                      o->terrain_position, o->terrain_normal, o->terrain_albedo, o->terrain_surface_id};
  ATM_CUDA(atm::launch_raster(M, S, layout_of(image), r->depth_key, O, float(near_m), float(tangent_half_fov),
                              view_mode, r->sm_count, static_cast<cudaStream_t>(stream)),
           "terrain raster");
  return ATM_OK;
}

ATM_API int atm_raster_emitted(const AtmRaster* r, int64_t* count, void* stream) {
  if (!r || !count) return fail(ATM_E_INVALID, "null argument");
  uint32_t v = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ATM_CUDA(cudaMemcpyAsync(&v, r->count, sizeof(v), cudaMemcpyDeviceToHost, s), "raster count");
  ATM_CUDA(cudaStreamSynchronize(s), "raster count");
  *count = int64_t(v);
  return ATM_OK;
}

// ---- ocean coverage ----------------------------------------------------------
struct AtmOcean {
  AtmOceanConfig config{};
  atm::OceanSpectrum spectrum{};
  double variances[atm::kOceanCascades] = {};
};

namespace {

// The spectrum's table (ocean.py:18-25) for the host-side (float64) set-up.
constexpr double kOceanPeriods[atm::kOceanCascades] = {2048.0, 256.0, 32.0};
constexpr double kOceanHeights[atm::kOceanCascades] = {0.62, 0.14, 0.025};
constexpr int kOceanModeX[12] = {3, 4, 4, 5, 5, 3, 2, 1, -1, -2, -3, -4};
constexpr int kOceanModeY[12] = {1, 1, 2, 1, 2, 2, 3, 4, 4, 3, 2, 1};
constexpr double kOceanWeights[12] = {1.0, 0.82, 0.72, 0.60, 0.52, 0.68, 0.55, 0.42, 0.36, 0.31, 0.27, 0.22};

double wind_amplitude_scale(const AtmOceanConfig& c) {  // _wind_amplitude_scale :232-233
  return std::min(std::max(c.wind_speed_mps / 8.0, 0.25), 2.0);
}

// Python's float modulo by a positive divisor: the result takes the
// divisor's sign (x % 1.0 lies in [0, 1)).
double py_mod1(double x) {
  double m = std::fmod(x, 1.0);
  if (m != 0.0) {
    if (m < 0.0) m += 1.0;
  } else {
    m = 0.0;
  }
  return m;
}

}  // namespace

ATM_API int atm_ocean_create(const AtmOceanConfig* config, AtmOcean** out) {
  if (!config || !out) return fail(ATM_E_INVALID, "null argument to atm_ocean_create");
  *out = nullptr;
  const AtmOceanConfig& c = *config;
  for (double a : c.albedo)
    if (!(a >= 0.0 && a <= 1.0)) return fail(ATM_E_INVALID, "ocean.albedo components must be in 0..1");
  if (!(c.normal_strength >= 0.0 && c.normal_strength <= 1.0))
    return fail(ATM_E_INVALID, "ocean.normal_strength must be in 0..1");
  if (!(c.max_visible_depth_m > 0.0) || !std::isfinite(c.max_visible_depth_m))
    return fail(ATM_E_INVALID, "ocean.max_visible_depth_m must be positive");
  if (c.spectrum_resolution != 32 && c.spectrum_resolution != 64 && c.spectrum_resolution != 128 &&
      c.spectrum_resolution != 256)
    return fail(ATM_E_INVALID, "ocean.spectrum_resolution must be 32, 64, 128 or 256");
  if (!(c.wind_speed_mps >= 0.1 && c.wind_speed_mps <= 40.0))
    return fail(ATM_E_INVALID, "ocean.wind_speed_mps must be in 0.1..40");
  if (!std::isfinite(c.wind_direction_degrees)) return fail(ATM_E_INVALID, "ocean.wind_direction_degrees must be finite");
  if (!(c.wave_height_scale >= 0.0 && c.wave_height_scale <= 4.0))
    return fail(ATM_E_INVALID, "ocean.wave_height_scale must be in 0..4");
  if (!(c.choppiness >= 0.0 && c.choppiness <= 1.0)) return fail(ATM_E_INVALID, "ocean.choppiness must be in 0..1");
  if (c.geometry_cascades < 0 || c.geometry_cascades > atm::kOceanCascades)
    return fail(ATM_E_INVALID, "ocean.geometry_cascades must be in 0..3");
  if (!(c.geometry_max_distance_m >= 0.0) || !std::isfinite(c.geometry_max_distance_m))
    return fail(ATM_E_INVALID, "ocean.geometry_max_distance_m must be non-negative");
  AtmOcean* o = new (std::nothrow) AtmOcean;
  if (!o) return fail(ATM_E_NOMEM, "host allocation failed");
  o->config = c;
  const int n = c.spectrum_resolution;
  const size_t texels = size_t(atm::kOceanCascades) * n * n;
  o->spectrum.n = n;
  cudaError_t e = cudaMalloc(&o->spectrum.height_gradient, texels * sizeof(float4));
  if (e == cudaSuccess) e = cudaMalloc(&o->spectrum.displacement, texels * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&o->spectrum.jacobian, texels * sizeof(float4));
  if (e == cudaSuccess) e = cudaMemset(o->spectrum.height_gradient, 0, texels * sizeof(float4));
  if (e == cudaSuccess) e = cudaMemset(o->spectrum.displacement, 0, texels * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemset(o->spectrum.jacobian, 0, texels * sizeof(float4));
  if (e != cudaSuccess) {
    atm_ocean_destroy(o);
    return e == cudaErrorMemoryAllocation ? fail(ATM_E_NOMEM, "ocean spectrum allocation failed")
                                          : cuda_fail(e, "ocean spectrum");
  }
  // per-cascade slope variance of the spectrum (_compute_slope_variance :235-258)
  double weight_sum = 0.0;
  for (double w : kOceanWeights) weight_sum += w;
  const double amplitude_scale = c.wave_height_scale * wind_amplitude_scale(c);
  for (int k = 0; k < atm::kOceanCascades; ++k) {
    double variance = 0.0;
    for (int m = 0; m < 12; ++m) {
      const double amplitude = kOceanHeights[k] * amplitude_scale * kOceanWeights[m] / weight_sum;
      const double wave_number = 2.0 * M_PI * std::hypot(double(kOceanModeX[m]), double(kOceanModeY[m])) /
                                 kOceanPeriods[k];
      const double slope = amplitude * wave_number;
      variance += 0.5 * (slope * slope);
    }
    o->variances[k] = variance;
  }
  *out = o;
  return ATM_OK;
}

ATM_API int atm_ocean_destroy(AtmOcean* o) {
  if (!o) return ATM_OK;
  if (o->spectrum.height_gradient) cudaFree(o->spectrum.height_gradient);
  if (o->spectrum.displacement) cudaFree(o->spectrum.displacement);
  if (o->spectrum.jacobian) cudaFree(o->spectrum.jacobian);
  delete o;
  return ATM_OK;
}

ATM_API int atm_ocean_rasterize(AtmOcean* o, const AtmOceanImages* im, const AtmImage* image, double planet_radius_m,
                                double camera_altitude_m, const double planet_frame[9], const double view_basis[9],
                                double tangent_half_fov, double time_seconds, int32_t debug_mode, void* stream) {
  if (!o || !im || !image || !planet_frame || !view_basis) return fail(ATM_E_INVALID, "null argument to atm_ocean_rasterize");
  if (image->width < 1 || image->height < 1 || (image->channels != 3 && image->channels != 4) ||
      image->stride_x <= 0 || image->stride_y <= 0)
    return fail(ATM_E_INVALID, "invalid AtmImage");
  if (!im->depth || !im->position || !im->normal || !im->albedo || !im->material_weights || !im->height_m ||
      !im->water_depth || !im->seabed_albedo || !im->seabed_normal || !im->slope_variance || !im->surface_id ||
      !im->cell_id)
    return fail(ATM_E_INVALID, "null G-buffer image");
  if (!(planet_radius_m > 0.0) || !std::isfinite(planet_radius_m) || !std::isfinite(camera_altitude_m) ||
      !(tangent_half_fov > 0.0) || !std::isfinite(tangent_half_fov) || !std::isfinite(time_seconds))
    return fail(ATM_E_INVALID, "planet radius, field of view and time must be finite (radius, fov positive)");
  for (int k = 0; k < 9; ++k)
    if (!std::isfinite(planet_frame[k]) || !std::isfinite(view_basis[k]))
      return fail(ATM_E_INVALID, "planet frame and view basis must be finite");
  const AtmOceanConfig& c = o->config;
  if (!c.surface_enabled) return ATM_OK;  // rasterize :709-710
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (c.enabled)
    ATM_CUDA(atm::launch_ocean_spectrum(o->spectrum, float(time_seconds), float(c.wave_height_scale *
                                                                                 wind_amplitude_scale(c)),
                                        float(c.choppiness), s),
             "ocean spectrum");
  const double wind = c.wind_direction_degrees * (M_PI / 180.0);  // math.radians
  atm::OceanFrame F{};
  F.radius = float(planet_radius_m);
  F.altitude = float(std::max(camera_altitude_m, 0.0));
  F.tf = float(tangent_half_fov);
  F.wind = float(wind);
  double max_displacement = 0.0;
  for (int k = 0; k < c.geometry_cascades; ++k) max_displacement += kOceanHeights[k];
  max_displacement = max_displacement * c.wave_height_scale * wind_amplitude_scale(c);
  F.max_displacement = float(c.enabled ? max_displacement : 0.0);
  F.geometry_max_distance = float(c.enabled ? c.geometry_max_distance_m : 0.0);
  F.normal_strength = float(c.normal_strength);
  F.max_visible_depth = float(c.max_visible_depth_m);
  for (int k = 0; k < 3; ++k) {
    F.east[k] = float(planet_frame[k]);
    F.up[k] = float(planet_frame[3 + k]);
    F.north[k] = float(planet_frame[6 + k]);
    F.right[k] = float(view_basis[k]);
    F.vup[k] = float(view_basis[3 + k]);
    F.fwd[k] = float(view_basis[6 + k]);
    F.albedo[k] = float(c.albedo[k]);
  }
  // texture offsets of the sea anchor below the camera (rasterize :709-726), float64
  const double cw = std::cos(wind), sw = std::sin(wind);
  static const double base[3][2][3] = {{{1, 0, 0}, {0, 0, 1}}, {{0, 1, 0}, {1, 0, 0}}, {{0, 0, 1}, {0, 1, 0}}};
  for (int k = 0; k < atm::kOceanCascades; ++k) {
    double au[3], av[3], du = 0.0, dvv = 0.0;
    for (int j = 0; j < 3; ++j) {
      au[j] = base[k][0][j] * cw + base[k][1][j] * sw;
      av[j] = -base[k][0][j] * sw + base[k][1][j] * cw;
    }
    for (int j = 0; j < 3; ++j) {
      const double anchor = planet_frame[3 + j] * planet_radius_m;
      du += anchor * au[j];
      dvv += anchor * av[j];
    }
    F.offsets[k][0] = float(py_mod1(du / kOceanPeriods[k]));
    F.offsets[k][1] = float(py_mod1(dvv / kOceanPeriods[k]));
    F.variances[k] = float(o->variances[k]);
  }
  F.geometry_cascades = c.geometry_cascades;
  F.enabled = c.enabled ? 1 : 0;
  F.debug_mode = debug_mode;
  atm::OceanImages G{im->depth,      im->position,      im->normal,        im->albedo,
                     im->material_weights, im->height_m, im->water_depth, im->seabed_albedo,
                     im->seabed_normal, im->slope_variance, im->surface_id, im->cell_id};
  ATM_CUDA(atm::launch_ocean_coverage(o->spectrum, F, layout_of(image), G, s), "ocean coverage");
  return ATM_OK;
}

ATM_API int atm_ocean_read_spectrum(AtmOcean* o, float* height, float* gradient, float* displacement, float* jacobian,
                                    void* stream) {
  if (!o) return fail(ATM_E_INVALID, "null ocean");
  const int n = o->spectrum.n;
  const size_t texels = size_t(atm::kOceanCascades) * n * n;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<float4> hg(texels), jac(texels);
  std::vector<float2> disp(texels);
  ATM_CUDA(cudaMemcpyAsync(hg.data(), o->spectrum.height_gradient, texels * sizeof(float4), cudaMemcpyDeviceToHost, s),
           "spectrum read");
  ATM_CUDA(cudaMemcpyAsync(disp.data(), o->spectrum.displacement, texels * sizeof(float2), cudaMemcpyDeviceToHost, s),
           "spectrum read");
  ATM_CUDA(cudaMemcpyAsync(jac.data(), o->spectrum.jacobian, texels * sizeof(float4), cudaMemcpyDeviceToHost, s),
           "spectrum read");
  ATM_CUDA(cudaStreamSynchronize(s), "spectrum read");
  for (size_t t = 0; t < texels; ++t) {
    if (height) height[t] = hg[t].x;
    if (gradient) gradient[2 * t] = hg[t].y, gradient[2 * t + 1] = hg[t].z;
    if (displacement) displacement[2 * t] = disp[t].x, displacement[2 * t + 1] = disp[t].y;
    if (jacobian)
      for (int k = 0; k < 4; ++k) jacobian[4 * t + k] = (&jac[t].x)[k];
  }
  return ATM_OK;
}
