/*
 * atm_capi.h - C ABI of the GB300 atmosphere path (LUT builds + per-pixel
 * composite).  Plain pointers, sizes and a cudaStream_t passed as void*; no
 * C++ or torch types.  Every entry point returns 0 on success or a negative
 * ATM_E* code; atm_last_error() gives the message of the calling thread's
 * last failure.  Every launch is stream-ordered on the caller's stream and
 * never synchronises the host, except where a function says so.
 *
 * Reference interface replaced: the Taichi class AtmosphereRenderer in
 * src/planet_renderer/atmosphere/renderer.py (constructor :51-116, update
 * :2072-2137, prepare_frame :2139-2187, composite :2189-2238,
 * set_luts_frozen :2057-2070) and its kernels _build_transmittance :1034,
 * _build_multi_scattering :1065, _build_sky_view :1208,
 * _build_aerial_perspective :1304, _prepare_surface_lighting :1422,
 * _composite :1827.  The Python layer (planet_renderer_gb300.atmosphere)
 * keeps that class's method names and argument meaning on top of this ABI.
 *
 * Conventions (reference renderer.py:44-49, renderer.py(top):1150):
 *  - vectors are in the camera's local East-Up-North frame; the camera is at
 *    the origin and the planet centre at (0, -camera_radius, 0);
 *  - position_view is the view-space (right, up, forward) hit position;
 *  - surface_id < 0 marks a sky pixel;
 *  - pixel (x, y) has screen_v = (y + 0.5) / height, increasing upward;
 *  - per-pixel images are addressed as base + (x*stride_x + y*stride_y)
 *    elements, each element `channels` floats (3 or 4).  The Taichi
 *    to_numpy() layout (W, H, 3) is stride_x = H, stride_y = 1, channels 3;
 *  - LUT read-back (atm_get_lut) is in the Taichi field layout (W, H[, D], 3).
 */
#ifndef ATM_CAPI_H
#define ATM_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes. */
#define ATM_OK 0
#define ATM_E_INVALID (-1)     /* bad argument: null pointer, size, range  */
#define ATM_E_CUDA (-2)        /* a CUDA call failed                        */
#define ATM_E_NOMEM (-3)       /* device allocation failed                  */
#define ATM_E_STATE (-4)       /* call order: e.g. composite before update  */
#define ATM_E_TIMEOUT (-5)     /* a bounded device wait gave up             */

/* Diagnostic views of the composite (reference diagnostics.py:15-25). */
#define ATM_VIEW_COMPOSITE 0
#define ATM_VIEW_SKY_VIEW 1
#define ATM_VIEW_CAMERA_TRANSMITTANCE 2
#define ATM_VIEW_TRANSMITTANCE_LUT 3
#define ATM_VIEW_MULTI_SCATTERING_LUT 4
#define ATM_VIEW_AERIAL_SCATTERING 5
#define ATM_VIEW_AERIAL_TRANSMITTANCE 6
#define ATM_VIEW_SURFACE_MASK 7
#define ATM_VIEW_AERIAL_FROXEL_ONLY 8
#define ATM_VIEW_AERIAL_DIRECT_ONLY 9
#define ATM_VIEW_AERIAL_BLEND_WEIGHT 10

/* LUT kinds for atm_get_lut. */
#define ATM_LUT_TRANSMITTANCE 0
#define ATM_LUT_MULTI_SCATTERING 1
#define ATM_LUT_SKY_VIEW 2
#define ATM_LUT_AERIAL 3

/*
 * Optical parameters and LUT quality of one spherical atmosphere.  Field for
 * field the reference's AtmosphereConfig (atmosphere/config.py:29-59); the
 * planet radius is passed per call, as in the reference.  Lengths in metres,
 * coefficients in 1/m.  Values are double, as Python floats are; kernels
 * round them to float exactly where the Taichi trace would.
 */
typedef struct AtmParams {
  double top_altitude_m;
  double rayleigh_scattering_per_m[3];
  double rayleigh_scale_height_m;
  double mie_scattering_per_m[3];
  double mie_extinction_per_m[3];
  double mie_scale_height_m;
  double mie_phase_g;
  double absorption_extinction_per_m[3];
  double absorption_peak_altitude_m;
  double absorption_half_width_m;
  double ground_albedo[3];
  int32_t transmittance_lut_width;
  int32_t transmittance_lut_height;
  int32_t multi_scattering_lut_width;
  int32_t multi_scattering_lut_height;
  int32_t sky_view_lut_width;
  int32_t sky_view_lut_height;
  int32_t aerial_lut_width;
  int32_t aerial_lut_height;
  int32_t aerial_lut_depth;
  int32_t transmittance_steps;
  int32_t multi_scattering_directions;
  int32_t multi_scattering_steps;
  int32_t sky_view_steps;
  int32_t aerial_steps_per_slice;
  int32_t aerial_horizon_raymarch_steps;
  int32_t aerial_terminator_substeps;
} AtmParams;

/* Addressing of the caller's per-pixel images (G-buffer, scene, space, hdr,
 * surface-lighting outputs).  All images of one call share it; surface_id
 * uses the same element strides with one int32 per element. */
typedef struct AtmImage {
  int32_t width;
  int32_t height;
  int64_t stride_x; /* elements between (x, y) and (x+1, y) */
  int64_t stride_y; /* elements between (x, y) and (x, y+1) */
  int32_t channels; /* floats per element of the float images: 3 or 4 */
} AtmImage;

/* Host-visible state of a renderer: the reference's public attributes
 * (atmosphere/renderer.py:97-116). has_* = 0 stands for Python None. */
typedef struct AtmState {
  int32_t luts_frozen;
  int32_t has_sky_snapshot;
  double sky_snapshot_altitude_m;
  double sky_snapshot_sun_cosine;
  int32_t has_aerial_snapshot;
  double aerial_snapshot_altitude_m;
  int64_t transmittance_rebuilds;
  int64_t multi_scattering_rebuilds;
  int64_t sky_view_rebuilds;
  int64_t aerial_rebuilds;
} AtmState;

/* Explicit inputs of one LUT build (atm_build_lut), bypassing the cache
 * keys of atm_update / atm_prepare_frame.  Angles in radians here. */
typedef struct AtmBuildArgs {
  double planet_radius_m;
  double camera_altitude_m;
  double sun_zenith_cosine;       /* sky-view                       */
  double sun_local[3];            /* aerial perspective             */
  double solar_irradiance[3];
  double sun_angular_radius_rad;
  double view_basis[9];           /* right, up, forward (aerial)    */
  double tangent_half_fov;        /* aerial                         */
  int32_t frame_width;            /* aerial: aspect = width/height  */
  int32_t frame_height;
} AtmBuildArgs;

typedef struct AtmHandle AtmHandle;

/* Message of the calling thread's last failed call ("" if none). */
const char* atm_last_error(void);

/* Allocate a renderer for width x height frames on the current CUDA device:
 * the four LUTs (zero-filled, as Taichi fields are) and a radiance-sample
 * counter.  Validates params with the reference's ranges
 * (atmosphere/config.py:61-128).  Replaces AtmosphereRenderer.__init__
 * (atmosphere/renderer.py:51-116). */
int atm_create(const AtmParams* params, int32_t width, int32_t height, AtmHandle** out);
int atm_destroy(AtmHandle* handle);

/* AtmosphereRenderer.set_luts_frozen (renderer.py:2057-2070). */
int atm_set_luts_frozen(AtmHandle* handle, int32_t frozen);
int atm_get_state(const AtmHandle* handle, AtmState* out);

/* AtmosphereRenderer.update (renderer.py:2072-2137): rebuild the
 * transmittance, multi-scattering and sky-view LUTs whose cache keys
 * changed; keys, float rounding points and counters as in the reference. */
int atm_update(AtmHandle* handle, double planet_radius_m, double camera_radius_m, const double sun_local[3],
               const double solar_irradiance[3], double sun_angular_radius_degrees, void* stream);

/* AtmosphereRenderer.prepare_frame (renderer.py:2139-2187): per surface
 * pixel sun transmittance and sky radiance into the caller's two images,
 * then the aerial-perspective volume unless frozen. view_basis = right, up,
 * forward (9 doubles). */
int atm_prepare_frame(AtmHandle* handle, const float* position_view, const int32_t* surface_id,
                      const AtmImage* image, double planet_radius_m, double camera_radius_m,
                      const double sun_local[3], const double solar_irradiance[3],
                      double sun_angular_radius_degrees, const double view_basis[9], double tangent_half_fov,
                      float* surface_sun_transmittance, float* surface_sky_radiance, void* stream);

/* AtmosphereRenderer.composite (renderer.py:2189-2238) -> hdr. */
int atm_composite(AtmHandle* handle, const float* scene_hdr, const float* space_hdr, const int32_t* surface_id,
                  const float* position_view, float* hdr, const AtmImage* image, double planet_radius_m,
                  double camera_radius_m, const double sun_local[3], const double solar_irradiance[3],
                  const double sun_disk_radiance[3], double sun_angular_radius_degrees,
                  const double view_basis[9], double tangent_half_fov, double star_contrast_start,
                  double star_contrast_end, int32_t diagnostic_view, void* stream);

/* Build one LUT from explicit inputs (no cache keys, counters untouched):
 * the kernels _build_transmittance :1034, _build_multi_scattering :1065,
 * _build_sky_view :1208, _build_aerial_perspective :1304. */
int atm_build_lut(AtmHandle* handle, int32_t kind, const AtmBuildArgs* args, void* stream);

/* Dimensions (w, h, d; d = 1 for 2-D) and device storage of a LUT: float4
 * texels, row-major [z][y][x]. */
int atm_lut_info(const AtmHandle* handle, int32_t kind, int32_t dims[3], void** device_ptr);

/* Copy a LUT to / from a device buffer in the Taichi field layout
 * (W, H[, D], 3) float32 - what the reference's field.to_numpy() holds. */
int atm_read_lut(const AtmHandle* handle, int32_t kind, float* dst_device, void* stream);
int atm_load_lut(AtmHandle* handle, int32_t kind, const float* src_device, void* stream);

/* Radiance samples (one constant-source segment each, reference
 * _scattering_segment :858-899) evaluated by composites since the last
 * reset.  Synchronises `stream`. */
int atm_read_sample_counter(AtmHandle* handle, int32_t reset, uint64_t* out, void* stream);

/* ---- batched LUT builds --------------------------------------------------
 * Many sky-view and aerial-perspective LUTs (time snapshots x cameras x
 * parameter sets, each with its own LUT size) built by one persistent
 * launch.  The reference builds one LUT per kernel launch
 * (renderer.py:1208 _build_sky_view, :1304 _build_aerial_perspective), each
 * job here computes exactly what one such launch computes. */
typedef struct AtmBatchJob {
  int32_t kind;            /* ATM_LUT_SKY_VIEW or ATM_LUT_AERIAL                   */
  int32_t param_set;       /* index into the sets given to atm_batch_create       */
  int32_t width;           /* LUT width  (sky-view 16..2048, aerial 4..256)       */
  int32_t height;          /* LUT height (sky-view 16..2048, aerial 4..256)       */
  int32_t depth;           /* aerial depth 8..256; 1 for sky-view                 */
  int32_t frame_width;     /* aerial: frame aspect = frame_width / frame_height   */
  int32_t frame_height;
  int32_t reserved;
  int64_t output_offset;   /* first float4 texel of this LUT in the output arena  */
  double camera_altitude_m;
  double sun_zenith_cosine; /* sky-view: f32-rounded key, as atm_update passes it */
  double sun_local[3];      /* aerial                                            */
  double view_basis[9];     /* aerial: right, up, forward                         */
  double tangent_half_fov;  /* aerial                                            */
} AtmBatchJob;

/* Work split of a batch launch (chosen by the Python autotuner). */
typedef struct AtmBatchTuning {
  int32_t sky_view_texels_per_item; /* 1..4096 */
  int32_t aerial_columns_per_item;  /* 1..4096 */
  int32_t blocks_per_sm;            /* 1..8 resident 256-thread blocks */
} AtmBatchTuning;

typedef struct AtmBatch AtmBatch;

/* Parameter sets of a batch with their planet radii; builds each set's
 * transmittance and multi-scattering LUTs (irradiance and sun size are
 * shared by all jobs, as the reference keys them). */
int atm_batch_create(const AtmParams* sets, const double* planet_radius_m, int32_t n_sets,
                     const double solar_irradiance[3], double sun_angular_radius_degrees, AtmBatch** out,
                     void* stream);
int atm_batch_destroy(AtmBatch* batch);
/* Build n_jobs LUTs into `arena` (device, arena_texels float4 texels; each
 * LUT row-major [z][y][x] at its output_offset) in one persistent launch.
 * The job table is uploaded to device memory owned by the batch (grown on
 * demand: the only allocations of this call). */
int atm_batch_build(AtmBatch* batch, const AtmBatchJob* jobs, int32_t n_jobs, void* arena, int64_t arena_texels,
                    const AtmBatchTuning* tuning, void* stream);
/* Radiance samples evaluated by batch builds since the last reset
 * (synchronises `stream`). */
int atm_batch_read_samples(AtmBatch* batch, int32_t reset, uint64_t* out, void* stream);
/* Device storage (float4 [y][x]) of a set's transmittance (kind 0) or
 * multi-scattering (kind 1) LUT. */
int atm_batch_static_lut(const AtmBatch* batch, int32_t param_set, int32_t kind, void** device_ptr);

/* ---- MLP surrogates --------------------------------------------------------
 * No counterpart in the reference (its atmosphere has no learned part): small
 * networks n_in -> [64 SiLU] x n_hidden -> n_out (n_in <= 16, n_out <= 8, 1-4
 * hidden layers) standing in for the sky-view
 * and aerial-perspective integrals.  Parameters live on the device as one
 * float array (per layer W (out x in, row-major) then b).  Training: fused
 * FP32 forward + backward of the mean squared error over the batch, Adam. */
typedef struct AtmMlp AtmMlp;
int atm_mlp_create(int32_t n_in, int32_t n_hidden_layers, int32_t n_out, uint64_t seed, AtmMlp** out);
int atm_mlp_destroy(AtmMlp* mlp);
int atm_mlp_info(const AtmMlp* mlp, int32_t* n_params, float** device_params);
int atm_mlp_reset_optimizer(AtmMlp* mlp, void* stream);
/* Device-to-device copies of the parameter array (checkpoint / restore). */
int atm_mlp_get_params(const AtmMlp* mlp, float* dst_device, void* stream);
int atm_mlp_set_params(AtmMlp* mlp, const float* src_device, void* stream);
/* Gradient of the batch loss into grad_out (device, n_params floats, may be
 * null) and the summed squared error into loss_out (device float, may be
 * null); parameters unchanged.  The loss is the mean over samples and
 * outputs of weight * (output - target)^2; weights (n x n_out, device) may be
 * null for all ones. */
int atm_mlp_gradient(AtmMlp* mlp, const float* inputs, const float* targets, const float* weights, int64_t n,
                     float* grad_out, float* loss_out, void* stream);
/* One Adam step on a batch (inputs n x n_in, targets and weights n x n_out,
 * device; weights may be null). */
int atm_mlp_train_step(AtmMlp* mlp, const float* inputs, const float* targets, const float* weights, int64_t n,
                       float lr, float beta1, float beta2, float eps, float* loss_out, void* stream);
/* Copy the current parameters into the BF16 tensor-core layout. */
int atm_mlp_pack_bf16(AtmMlp* mlp, void* stream);
/* outputs (n x n_out) = network(inputs); precision 0 = FP32 CUDA cores,
 * 1 = BF16 tensor cores (mma.sync) with FP32 accumulation, 2 = BF16 on the
 * 5th-generation tensor cores (tcgen05.mma, accumulators in tensor memory);
 * 1 and 2 after atm_mlp_pack_bf16.  Precision 2 synchronises `stream` and
 * returns ATM_E_TIMEOUT if an MMA did not complete in time. */
int atm_mlp_forward(const AtmMlp* mlp, const float* inputs, float* outputs, int64_t n, int32_t precision,
                    void* stream);

/* ---- learned surrogates ----------------------------------------------------
 * No counterpart in the reference.  Feature vectors, every entry in [-1, 1]:
 *   0     altitude h of the segment's first point inside the shell,
 *         2 sqrt(h / top) - 1
 *   1     view zenith there in the sky-view v mapping (renderer.py
 *         :482-520), 2 v - 1
 *   2     sun cosine there in the multi-scattering u mapping (:522-568),
 *         2 u - 1
 *   3     cosine of the relative azimuth of view and sun about the vertical
 *   4, 5  Rayleigh / Mie scale height,
 *         2 (ln H - ln H_min) / (ln H_max - ln H_min) - 1
 *   6     aerial only: segment length, 2 ln(clamp(len, 1 m, 2000 km)) /
 *         ln(2000 km) - 1
 *   7, 8  aerial only: sun cosine (as 2) and altitude (as 0, clamped to
 *         [0, top]) at the segment's end
 *   9, 10 aerial only: the same at the segment's middle
 *   6, 7  sky only: sun cosine and altitude (as 7, 8) where the sky-view march
 *         ends (the shell top or the ground)
 *   8, 9  sky only: the same at the march's lowest point (the closest
 *         approach to the planet's centre, clamped to the march)
 * Targets: sky (ATM_SURROGATE_SKY) ln(L / E + 1e-7) per channel of the sky
 * radiance along the ray (the sky-view march, :1208-1302, from the ray's
 * altitude); aerial (ATM_SURROGATE_AERIAL) the same for the in-scattering of
 * the segment (the limb integrator, :1667-1755), then its optical depth per
 * channel (-ln of :1603-1665, capped at 30). */
#define ATM_SURROGATE_SKY 0
#define ATM_SURROGATE_AERIAL 1

/* Training samples computed by the plain integrator over the parameter sets
 * of a batch (their transmittance and multi-scattering LUTs; the sets must
 * share the planet radius and the shell top).  Features are uniform over the
 * box above, drawn per sample index from `seed` (sample i does not depend on
 * n), the parameter set uniform among the batch's.  scale_height_range:
 * H_R min, max, H_M min, max in metres.  features: n x 10 (sky) or n x 11
 * (aerial) floats, targets n x 3 or n x 6, device.  options (aerial kind,
 * may be null for uniform sampling) concentrate samples where surface pixels
 * need them. */
typedef struct AtmSampleOptions {
  double shell_top_fraction; /* share of segments starting at the shell top (feature 0 = 1),
                                where every segment seen from above the shell starts   */
  double surface_fraction;   /* share of segments ending at an altitude uniform in
                                [surface_min_m, surface_max_m] (where the ray reaches it) */
  double surface_min_m;
  double surface_max_m;
  double start_min_m;        /* segments start at an altitude in [start_min_m, start_max_m]
                                (uniform in the altitude feature) when start_min_m <
                                start_max_m; otherwise anywhere in the shell           */
  double start_max_m;
  double sun_angle_fraction;    /* share of samples whose sun zenith at the start is uniform in
                                   angle in [0, sun_angle_max_degrees] (the rest uniform in the
                                   sun feature, which concentrates on the horizon)          */
  double sun_angle_max_degrees;
} AtmSampleOptions;
int atm_surrogate_samples(AtmBatch* batch, int32_t kind, int64_t n, uint64_t seed, const AtmSampleOptions* options,
                          const double scale_height_range[4], float* features, float* targets, void* stream);

/* Networks and error check of atm_composite_surrogate. */
typedef struct AtmSurrogate {
  const AtmMlp* aerial;  /* 11 -> 4 x 64 -> 6, packed (atm_mlp_pack_bf16), or null:
                            plain integrator for every surface pixel            */
  const AtmMlp* sky;     /* 10 -> 3 x 64 -> 3, packed, or null: sky-view LUT    */
  const AtmMlp* aerial_above_shell; /* 11 -> 4 x 64 -> 6 used instead of aerial
                            when the camera is above the shell (every segment
                            then starts at the shell top), or null            */
  double scale_height_range[4];   /* of features 4, 5 (as in training)          */
  double trained_planet_radius_m; /* the networks' planet; the frame must match */
  double trained_top_altitude_m;
  double check_fraction; /* share of MLP pixels re-integrated by the plain path */
  double aerial_floor;   /* the aerial network's radiance outputs are
                            ln(L / E + aerial_floor + aerial_floor_t T), T the
                            segment's transmittance from the LUT ...          */
  double aerial_floor_t;
  double sky_floor;      /* ... and the sky network's ln(L / E + sky_floor)    */
  double twilight_cosine; /* gate: |sun cosine| below this at a surface
                            segment's start, middle or end -> plain path     */
  double sky_twilight_cosine; /* gate: |sun cosine| at the camera below this ->
                            sky pixels read the sky-view LUT (e.g. 0.1)       */
  double limb_degrees;   /* gate: view ray within this of the limb (e.g. 0.5) */
  uint32_t seed;         /* picks the checked pixels                            */
  int32_t tc_wait_polls; /* bound of each tensor-core completion wait, in
                            mbarrier polls: 0 = the library's bound (2^20
                            polls, far beyond any MMA's latency); -1 = no
                            poll, every wait gives up at once (exercises the
                            timeout path: every MLP pixel then takes the plain
                            path); other values as given                       */
  float* stats;          /* device float[8] accumulated into, or null: checked
                            pixels, sum and max of their relative error, gated
                            surface pixels, MLP surface pixels, MLP sky pixels,
                            sky-view-LUT sky pixels, 128-pixel tiles whose
                            tensor-core MMA did not complete in time (0)       */
  int32_t gate_terminator; /* non-zero: a surface segment whose sun cosine has
                            different signs at its start, middle and end (it
                            crosses the terminator) takes the plain path too */
  int32_t calibration_tile; /* 0: off.  Else the side (a power of two, 16..256
                            pixels) of the calibration tiles: the checked
                            pixels' log ratio of the plain path's in-scattering
                            to the network's, averaged per tile (clamped to
                            +-0.3; tiles with at least 4 checked pixels),
                            rescales the network's in-scattering of the
                            tile's other MLP pixels.  Costs a width x height x
                            3 float scratch image (allocated on first use) and
                            one extra pass over the frame.                  */
} AtmSurrogate;

/* COMPOSITE view of atm_composite with the per-pixel limb integrator replaced
 * by the aerial network and the sky-view lookup by the sky network (BF16 on
 * the 5th-generation tensor cores, tcgen05.mma, FP32 accumulators in tensor
 * memory).  Surface pixels keep the plain path's
 * transmittance (the two-tap LUT ratio of :1603-1665); the network gives
 * their in-scattering.  The plain integrator remains the
 * per-pixel fallback where a gate trips (view ray within limb_degrees of the
 * limb; for surface pixels the sun cosine below twilight_cosine at the
 * segment's start, middle or end; for sky pixels the camera's sun cosine
 * below sky_twilight_cosine or the camera above the shell), and re-integrates
 * check_fraction of the MLP pixels, whose error goes to stats; those pixels
 * keep the plain result.  A 128-pixel tile whose tensor-core MMA does not
 * complete within the wait bound gives its MLP pixels to the plain path (the
 * frame stays correct) and sets the handle's timeout flag, which atm_check
 * reports.  Allocates the handle's fallback queue (4 bytes a pixel) on first
 * use; stream-ordered and capturable afterwards. */
int atm_composite_surrogate(AtmHandle* handle, const float* scene_hdr, const float* space_hdr,
                            const int32_t* surface_id, const float* position_view, float* hdr, const AtmImage* image,
                            double planet_radius_m, double camera_radius_m, const double sun_local[3],
                            const double solar_irradiance[3], const double sun_disk_radiance[3],
                            double sun_angular_radius_degrees, const double view_basis[9], double tangent_half_fov,
                            double star_contrast_start, double star_contrast_end, const AtmSurrogate* surrogate,
                            void* stream);

/* Sky radiance of every pixel along its own view ray from the camera (the
 * learned sky-view workload; no G-buffer: every pixel is treated as sky),
 * written to the first three floats of each `radiance` element:
 *  ATM_SKY_PIXELS_PLAIN  the plain integrator per pixel: the sky-view LUT's
 *                        march (:1208-1302, sky_view_steps warped segments)
 *                        along the pixel's ray;
 *  ATM_SKY_PIXELS_NET    the sky network of `surrogate` (BF16 on tcgen05), the
 *                        plain integrator where a gate trips (|sun cosine|
 *                        at the camera below sky_twilight_cosine, the ray
 *                        within limb_degrees of the limb, the camera above
 *                        the shell) or a tensor-core wait gives up (which
 *                        sets the flag atm_check reports);
 *  ATM_SKY_PIXELS_LUT    the reference's path: a bilinear tap of the sky-view
 *                        LUT (:1474-1525) built by atm_update.
 * Plain pixels add their samples to the radiance-sample counter.  No
 * counterpart in the reference, whose sky is the LUT path only. */
#define ATM_SKY_PIXELS_PLAIN 0
#define ATM_SKY_PIXELS_NET 1
#define ATM_SKY_PIXELS_LUT 2
int atm_sky_pixels(AtmHandle* handle, int32_t mode, float* radiance, const AtmImage* image, double planet_radius_m,
                   double camera_radius_m, const double sun_local[3], const double solar_irradiance[3],
                   double sun_angular_radius_degrees, const double view_basis[9], double tangent_half_fov,
                   const AtmSurrogate* surrogate, void* stream);

/* Synchronises `stream` and reports, then clears, the device-side errors of
 * the handle's earlier stream-ordered calls: ATM_E_TIMEOUT when a
 * tensor-core wait of atm_composite_surrogate gave up since the last check
 * (those pixels took the plain path), ATM_OK otherwise.  No counterpart in
 * the reference, whose kernels have no bounded waits. */
int atm_check(AtmHandle* handle, void* stream);

/* COMPOSITE view of atm_composite that allocates nothing.  No counterpart in
 * the reference.  For callers that may not call cudaMalloc: an engine or
 * plugin host that owns every device allocation through its own pool, a
 * real-time frame loop where an allocation's implicit synchronisation and
 * latency are not acceptable, a process running under a fixed device-memory
 * budget.  Everything is caller-owned: the transmittance, multi-scattering
 * and sky-view LUTs (device buffers of float4 texels, row-major [y][x], with
 * the sizes in `params`, as atm_lut_info describes them), the images and
 * `samples_out` (device, may be null).  The only scratch is a fixed array of
 * 65,536 per-tile sample counts (256 KB) inside the library; every GPU that
 * loads the library holds it until the process exits.  Frames needing more
 * than 65,536 16x16 tiles (16.7 million pixels) are rejected with
 * ATM_E_INVALID.  The first call on each device looks the array's address up
 * (cudaGetSymbolAddress) with that device current: make that first call
 * before any stream capture.  All calls share the array: calls that overlap
 * on the GPU (other streams, other threads) race on it and may report wrong
 * sample counts.  Each call writes every tile slot it later sums, so nothing
 * needs clearing between calls.  sky_lut_camera_altitude_m is the altitude
 * the sky-view LUT was built for (atm_update's f32-rounded key).  Writes hdr
 * and, when samples_out is set, the frame's radiance-sample count. */
int atm_composite_noalloc(const AtmParams* params, const void* transmittance_lut, const void* multi_scattering_lut,
                          const void* sky_view_lut, const float* scene_hdr, const float* space_hdr,
                          const int32_t* surface_id, const float* position_view, float* hdr, const AtmImage* image,
                          double planet_radius_m, double camera_radius_m, double sky_lut_camera_altitude_m,
                          const double sun_local[3], const double solar_irradiance[3],
                          const double sun_disk_radiance[3], double sun_angular_radius_degrees,
                          const double view_basis[9], double tangent_half_fov, double star_contrast_start,
                          double star_contrast_end, uint64_t* samples_out, void* stream);

/* ---- display post-process -------------------------------------------------
 * PostProcessor (src/planet_renderer/postprocess.py:75-207), the step after
 * the atmosphere stage: bloom at half resolution (2x2 extract with the soft
 * threshold and bright-pass cap, then separable 5-tap blur passes) and the
 * display transform (exposure, bilinear bloom, ACES fit, sRGB).  The bloom
 * planes are allocated at creation; atm_post_process is stream-ordered and
 * capturable. */
typedef struct AtmPostConfig { /* PostprocessConfig, postprocess.py:10-38 */
  double exposure_ev;     /* finite, [-20, 20]; validated only: atm_post_process takes the EV */
  double bloom_threshold; /* finite, >= 0 */
  double bloom_knee;      /* finite, >= 0 */
  double bloom_clamp;     /* finite, >= 0 */
  double bloom_strength;  /* finite, >= 0 */
  int32_t bloom_passes;   /* 0..8 */
} AtmPostConfig;
typedef struct AtmPost AtmPost;
/* PostProcessor.__init__ (:78-86) with PostprocessConfig's validation
 * (:21-38): ATM_E_INVALID with the reference's message on a bad field. */
int atm_post_create(const AtmPostConfig* config, int32_t width, int32_t height, AtmPost** out);
int atm_post_destroy(AtmPost* post);
/* PostProcessor.process (:176-207): hdr -> display, both with `image`'s
 * shape and strides (3 or 4 floats per pixel; display's first three are
 * written, hdr is not modified).  Exposure 2^exposure_ev applies only when
 * tone_map != 0; bloom runs when bloom != 0 and the configuration has
 * passes and strength. */
int atm_post_process(AtmPost* post, const float* hdr, float* display, const AtmImage* image, double exposure_ev,
                     int32_t bloom, int32_t tone_map, void* stream);
/* The half-resolution bloom plane of the last atm_post_process that ran
 * bloom (dims: half width, half height), copied stream-ordered into
 * dst_device (float4 [y][x], dims[0] * dims[1] texels; may be null to query
 * dims), for inspection. */
int atm_post_read_bloom(const AtmPost* post, int32_t dims[2], float* dst_device, void* stream);

/* ---- surface shading -----------------------------------------------------
 * PlanetRenderer._shade_surface (src/planet_renderer/renderer.py:1277-1575),
 * the consumer of atm_prepare_frame's surface_sun_transmittance and
 * surface_sky_radiance: Lambertian land; ocean pixels (advanced ocean on) with
 * a GGX-style sun specular, Fresnel sky reflection and a water body over a
 * seabed reconstructed along the refracted view ray from the opaque terrain
 * snapshot.  Arguments as the reference kernel's (rounded to float32). */
typedef struct AtmShadeParams {
  double sun_global[3];
  double solar_irradiance[3];
  double view_right_global[3];
  double view_up_global[3];
  double view_forward_global[3];
  int32_t advanced_ocean_enabled;
  int32_t mode; /* 0 lit; otherwise albedo (the debug views) */
  double ocean_roughness;
  double ocean_f0;
  double ocean_sky_strength;
  double ocean_absorption[3];
  double ocean_scattering[3];
  double ocean_max_depth;
  double ocean_refraction_index;
  double ocean_refraction_strength;
  double ocean_refraction_max_offset_pixels;
  double sun_angular_radius; /* radians */
  double tangent_half_fov;
  int32_t ocean_surface_id; /* OCEAN_SURFACE_ID (ocean.py:17) */
  int32_t reserved;
} AtmShadeParams;
/* Device images, all of `image`'s shape and element strides: float images
 * with image->channels floats per element (the first three read or written),
 * water_depth and slope_variance one float, the ids one int32. */
typedef struct AtmShadeImages {
  const float* position;       /* view space (gbuffer_position) */
  const float* normal;         /* global frame (gbuffer_normal) */
  const float* albedo;
  const float* water_depth;    /* gbuffer_water_depth_m */
  const float* seabed_albedo;
  const float* seabed_normal;
  const float* slope_variance; /* gbuffer_ocean_slope_variance */
  const int32_t* surface_id;
  const float* terrain_position; /* the opaque terrain snapshot */
  const float* terrain_normal;
  const float* terrain_albedo;
  const int32_t* terrain_surface_id;
  const float* sun_transmittance; /* atm_prepare_frame outputs */
  const float* sky_radiance;
  float* surface_hdr;             /* output */
} AtmShadeImages;
int atm_shade_surface(const AtmShadeParams* params, const AtmShadeImages* images, const AtmImage* image,
                      void* stream);

/* The frame's last three steps in one pass over the pixels: the surface
 * lighting of atm_prepare_frame (:1422-1472), the surface shading of
 * atm_shade_surface (renderer.py:1277-1575) and the COMPOSITE view of
 * atm_composite (or, with `surrogate`, of atm_composite_surrogate), as the
 * reference's frame calls them in sequence (renderer.py:1671-1727).  Each
 * pixel's lighting and shaded colour stay in registers: the three
 * full-resolution images the separate calls write and read back
 * (surface_sun_transmittance, surface_sky_radiance, surface_hdr) are not
 * formed, and `images`' sun_transmittance, sky_radiance and surface_hdr may
 * be null.  The aerial-perspective volume of prepare_frame (which the
 * COMPOSITE view does not read) is not rebuilt.  Needs the LUTs of a
 * preceding atm_update.  No counterpart in the reference. */
int atm_render_frame(AtmHandle* handle, const AtmShadeParams* shade, const AtmShadeImages* images,
                     const float* space_hdr, float* hdr, const AtmImage* image, double planet_radius_m,
                     double camera_radius_m, const double sun_local[3], const double solar_irradiance[3],
                     const double sun_disk_radiance[3], double sun_angular_radius_degrees, const double view_basis[9],
                     double tangent_half_fov, double star_contrast_start, double star_contrast_end,
                     const AtmSurrogate* surrogate, void* stream);

/* ---- terrain raster: the G-buffer producer ----------------------------------
 * PlanetRenderer's terrain raster (src/planet_renderer/renderer.py :628-1269),
 * the step before the atmosphere stage: _clip (back-face culling of surface
 * triangles, skirts double-sided, trivial reject, Sutherland-Hodgman against
 * the near plane and the frustum sides), _emit (projection snapped to 1/256
 * pixel, edge equations, top-left rule), _raster_depth_direct (an atomic
 * 64-bit minimum of depth bits << 32 | triangle per covered pixel centre) and
 * _resolve_raster with _surface_color (perspective-correct attributes of the
 * nearest triangle, the albedo of the view mode).  The patches' vertex
 * streams are the camera-view-space output of the terrain's LOD system,
 * which is not part of this library. */
typedef struct AtmRasterMesh {
  const float* view;        /* [patches][vertices_per_patch][3] view space (right, up, forward), m */
  const float* normal;      /* [patches][vertices_per_patch][3] */
  const float* material;    /* [patches][vertices_per_patch][4] material weights */
  const float* height_m;    /* [patches][vertices_per_patch] terrain height */
  const int32_t* cell;      /* [patches][vertices_per_patch] cell ids */
  const int32_t* triangles; /* [triangles_per_patch][3] vertex indices within a patch: the
                               surface triangles, then the skirts (4 edges x 2 resolution) */
  const int32_t* active_slots; /* [n_active] the patches (slots) to draw, in order */
  const int32_t* skirt_mask;   /* [patches] bit e enables skirt edge e, or null: no skirts */
  const int32_t* slot_level;   /* [patches] LOD level (view mode 2), or null */
  int32_t patches, vertices_per_patch, triangles_per_patch, surface_triangles_per_patch;
  int32_t resolution;          /* cells per patch side (2 resolution skirt triangles per edge) */
  int32_t n_active;
} AtmRasterMesh;
/* Device G-buffer images sharing `image`'s shape and element strides:
 * position (view space), normal, albedo with image->channels floats per
 * element, material_weights 4 floats, depth and height_m one float,
 * surface_id and cell_id one int32.  Uncovered pixels get surface_id = -1
 * and cell_id = -1; their other values are left as they were (as the
 * reference leaves them). */
typedef struct AtmRasterOutputs {
  float* depth;
  float* position;
  float* normal;
  float* albedo;
  float* material_weights;
  float* height_m;
  int32_t* surface_id;
  int32_t* cell_id;
  /* The opaque terrain snapshot the ocean shading reads
   * (_snapshot_terrain_gbuffer, renderer.py:1270-1275), written in the same
   * pass; null terrain_surface_id skips it.  Uncovered pixels get
   * terrain_surface_id = -1 (the other snapshot values are not read there). */
  float* terrain_position;
  float* terrain_normal;
  float* terrain_albedo;
  int32_t* terrain_surface_id;
} AtmRasterOutputs;
typedef struct AtmRaster AtmRaster;
/* PlanetRenderer's raster buffers (renderer.py:200-236): the emitted-triangle
 * stream (max_patches x triangles_per_patch x 6 triangles) and the depth keys
 * of a width x height frame. */
int atm_raster_create(int32_t width, int32_t height, int32_t max_patches, int32_t triangles_per_patch,
                      AtmRaster** out);
int atm_raster_destroy(AtmRaster* raster);
/* _clip + _raster_depth_direct + _resolve_raster of one frame (view_mode: 0
 * lit albedo, 1 height bands, 2 LOD-level hue, 3 patch hash; renderer.py
 * :1008-1058).  Stream-ordered; allocates nothing. */
int atm_raster_terrain(AtmRaster* raster, const AtmRasterMesh* mesh, double near_m, double tangent_half_fov,
                       int32_t view_mode, const AtmRasterOutputs* outputs, const AtmImage* image, void* stream);
/* Triangles the last atm_raster_terrain emitted (clipped_count; synchronises
 * `stream`).  More than the stream's capacity means some were dropped, as
 * the reference drops them. */
int atm_raster_emitted(const AtmRaster* raster, int64_t* count, void* stream);

/* ---- ocean coverage: the sea-level part of the G-buffer -----------------------
 * OceanRenderer (src/planet_renderer/ocean.py:193-771): per frame the
 * directional wave spectrum (_build_directional_spectrum :260-337, three
 * periodic cascades) and the coverage pass (_rasterize :517-684): each view
 * ray against the sea-level sphere, near-field wave geometry by fixed-point
 * sphere solves, and where the sea is nearer than the terrain the water
 * surface's G-buffer values (view position, footprint-filtered wave normal,
 * slope variance, seabed colour / normal / water depth from the terrain pixel
 * it covers, surface_id = OCEAN_SURFACE_ID, cell_id = -1). */
typedef struct AtmOceanConfig { /* OceanConfig's fields the pass reads (ocean.py:38-110) */
  int32_t surface_enabled;      /* 0: the pass writes nothing */
  int32_t enabled;              /* advanced waves; 0: flat sea level, no spectrum */
  double albedo[3];
  double normal_strength;       /* 0..1 */
  double max_visible_depth_m;   /* > 0 */
  int32_t spectrum_resolution;  /* 32, 64, 128 or 256 */
  int32_t geometry_cascades;    /* 0..3 */
  double wind_speed_mps;        /* 0.1..40 */
  double wind_direction_degrees;
  double wave_height_scale;     /* 0..4 */
  double choppiness;            /* 0..1 */
  double geometry_max_distance_m; /* >= 0 */
} AtmOceanConfig;
/* Device G-buffer images sharing `image`'s shape and element strides:
 * position (view space), normal, albedo, seabed_albedo and seabed_normal
 * with image->channels floats per element, material_weights 4 floats, the
 * rest one value.  Read where the terrain was drawn (surface_id >= 0), and
 * overwritten at the pixels the sea covers. */
typedef struct AtmOceanImages {
  float* depth;
  float* position;
  float* normal;
  float* albedo;
  float* material_weights;
  float* height_m;
  float* water_depth;
  float* seabed_albedo;
  float* seabed_normal;
  float* slope_variance;
  int32_t* surface_id;
  int32_t* cell_id;
} AtmOceanImages;
typedef struct AtmOcean AtmOcean;
/* OceanRenderer.__init__ (:197-230): validates the configuration and
 * allocates the spectrum (3 cascades x resolution^2 texels). */
int atm_ocean_create(const AtmOceanConfig* config, AtmOcean** out);
int atm_ocean_destroy(AtmOcean* ocean);
/* OceanRenderer.rasterize (:686-762) after PlanetRenderer's terrain raster
 * (renderer.py:1643-1663): planet_frame = (east, up, north) of the camera's
 * local frame in planet coordinates, view_basis = (right, up, forward) in the
 * local frame, 9 doubles each.  Stream-ordered; allocates nothing. */
int atm_ocean_rasterize(AtmOcean* ocean, const AtmOceanImages* images, const AtmImage* image, double planet_radius_m,
                        double camera_altitude_m, const double planet_frame[9], const double view_basis[9],
                        double tangent_half_fov, double time_seconds, int32_t debug_mode, void* stream);
/* The last frame's spectrum copied to host memory (tests; synchronises):
 * each array is [3][resolution][resolution] (cascade, x, y) of 1, 2, 2 and
 * 4 floats: height, gradient, displacement, displacement Jacobian.  Any
 * pointer may be null. */
int atm_ocean_read_spectrum(AtmOcean* ocean, float* height, float* gradient, float* displacement, float* jacobian,
                            void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ATM_CAPI_H */
