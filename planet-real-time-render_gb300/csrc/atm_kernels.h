// atm_kernels.h - host-side launch wrappers of the atmosphere kernels.
// Internal to libplanet_atm; the public interface is include/atm_capi.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "atm_capi.h"
#include "atm_device.cuh"

namespace atm {

DevParams make_dev_params(const AtmParams& p);

// Per-pixel image addressing: element (x, y) at base + (x*sx + y*sy)*channels.
struct ImageLayout {
  int32_t width, height;
  int64_t sx, sy;
  int32_t channels;
};

struct CompositeScalars {
  float bottom, cam_alt, sky_alt, ar, tanfov, star_start, star_end;
  float sun[3], E[3], disk[3], right[3], up[3], fwd[3];
  int32_t view;
};

cudaError_t launch_transmittance(const DevParams& P, float bottom, float4* out, cudaStream_t s);
// The LUT builds and the composite add the radiance samples they evaluate to
// `counter` (may be null).
cudaError_t launch_multi_scattering(const DevParams& P, float bottom, const float E[3], float ar,
                                    const float4* tlut, float4* out, unsigned long long* counter, cudaStream_t s);
cudaError_t launch_sky_view(const DevParams& P, float bottom, float cam_alt, float sun_cos, const float E[3],
                            float ar, const float4* tlut, const float4* mslut, float4* out,
                            unsigned long long* counter, cudaStream_t s);
cudaError_t launch_aerial(const DevParams& P, int width, int height, float bottom, float cam_alt, const float sun[3],
                          const float E[3], float ar, const float right[3], const float up[3], const float fwd[3],
                          float tanfov, const float4* tlut, const float4* mslut, float4* out,
                          unsigned long long* counter, cudaStream_t s);
cudaError_t launch_prepare_surface(const DevParams& P, const ImageLayout& L, const float* pos, const int32_t* sid,
                                   float bottom, float cam_alt, const float sun[3], float ar, const float right[3],
                                   const float up[3], const float fwd[3], const float4* tlut, const float4* mslut,
                                   float* out_sun_t, float* out_sky, cudaStream_t s);
cudaError_t launch_composite(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                             const float* scene, const float* space, const int32_t* sid, const float* pos,
                             const float4* tlut, const float4* mslut, const float4* svlut, const float4* aplut,
                             float* hdr, unsigned long long* sample_counter, cudaStream_t s);
// LUT (float4 [z][y][x]) -> Taichi field layout (W, H[, D], 3) floats.
cudaError_t launch_lut_to_fields(const float4* lut, int w, int h, int d, float* dst, cudaStream_t s);
// Taichi field layout (W, H[, D], 3) floats -> LUT (float4 [z][y][x]).
cudaError_t launch_fields_to_lut(const float* src, int w, int h, int d, float4* lut, cudaStream_t s);

// Batched builds (atm_batch.cu): opaque device job descriptors.
struct BatchJobDev;
size_t batch_job_size();
void fill_batch_job(BatchJobDev& d, const DevParams& set_params, const AtmBatchJob& j, float4* arena,
                    const float4* tlut, const float4* mslut, double radius, const double E[3], double ar_rad,
                    int per_item);
cudaError_t launch_batch(const BatchJobDev* jobs, const long long* prefix, int n_jobs, long long n_items,
                         unsigned long long* ticket, unsigned long long* samples, int blocks, cudaStream_t s);

// MLP surrogates (atm_mlp.cu): n_in -> [64 SiLU] x (n_layers - 1) -> n_out.
constexpr int kMaxMlpLayers = 5;
struct MlpShape {
  int n_in, n_out, n_layers, n_params;
  int in_dim[kMaxMlpLayers], out_dim[kMaxMlpLayers], off_w[kMaxMlpLayers], off_b[kMaxMlpLayers];
};
MlpShape make_mlp_shape(int n_in, int n_hidden, int n_out);
int mlp_train_ctas(long long n);
size_t mlp_train_smem_bytes(const MlpShape& m);
size_t mlp_bf16_bytes(const MlpShape& m);
// weights: per (sample, output) factors of the squared error, or null
cudaError_t launch_mlp_grad(const MlpShape& m, const float* params, const float* inputs, const float* targets,
                            const float* weights, long long n, float* grad_partial, float* loss_partial, float* grad,
                            cudaStream_t s);
cudaError_t launch_reduce_partials(const float* partial, int rows, int cols, float* out, cudaStream_t s);
cudaError_t launch_adam(float* params, const float* grad, float* m1, float* m2, int n, float lr, float b1, float b2,
                        float eps, long long step, cudaStream_t s);
cudaError_t launch_mlp_forward_f32(const MlpShape& m, const float* params, const float* inputs, float* outputs,
                                   long long n, cudaStream_t s);
cudaError_t launch_mlp_pack_bf16(const MlpShape& m, const float* params, void* packed, cudaStream_t s);
// tcgen05 path: packed layout of atm_mlp_tc.cuh; *error set if an MMA timed out
size_t mlp_tc_bytes(const MlpShape& m);
cudaError_t launch_mlp_pack_tc(const MlpShape& m, const float* params, void* packed, cudaStream_t s);
cudaError_t launch_mlp_forward_tc(const MlpShape& m, const void* packed, const float* inputs, float* outputs,
                                  long long n, int* error, int sm_count, cudaStream_t s);
cudaError_t launch_mlp_forward_bf16(const MlpShape& m, const void* packed, const float* inputs, float* outputs,
                                    long long n, int sm_count, cudaStream_t s);

// Surrogates (atm_surrogate.cu).  Targets: log(L / E + floor) and optical
// depth; segment lengths up to 2000 km.
constexpr float kSurrogateFloor = 1.0e-7f;
constexpr float kSurrogateMaxLength = 2.0e6f;
constexpr float kSurrogateMaxDepth = 30.0f;
constexpr int kSurrogateApIn = 11, kSurrogateApOut = 6, kSurrogateApHidden = 4;
constexpr int kSurrogateSkyIn = 10, kSurrogateSkyOut = 3, kSurrogateSkyHidden = 3;
struct SurrogateSetDev {
  DevParams P;
  const float4* tlut;
  const float4* mslut;
  float bottom;
  float lhr_n, lhm_n;  // normalised log scale heights (features 4, 5)
};
// Bound of a tensor-core completion wait, in mbarrier polls (each try_wait
// itself suspends for a bounded time): far beyond any MMA's latency.
constexpr int kTcWaitTries = 1 << 20;

struct SurrogateNets {
  const unsigned char* ap;   // packed BF16 aerial network (11 -> 4x64 -> 6) or null
  const unsigned char* sky;  // packed BF16 sky network (10 -> 3x64 -> 3) or null
  int ap_bytes, sky_bytes;   // multiples of 16
  float lhr_n, lhm_n;        // the frame's normalised log scale heights
  float floor, floor_t;      // aerial output: ln(L / E + floor + floor_t T)
  float sky_floor;           // sky output: ln(L / E + sky_floor)
  float twilight_cos;        // gate: |sun cosine| at a surface segment below this -> plain path
  float sky_twilight_cos;    // gate: |sun cosine| at the camera below this -> sky-view LUT
  float limb_rad;            // gate: view ray within this of the limb -> plain path
  int wait_tries;            // bound of each tensor-core completion wait (mbarrier polls)
  int gate_crossing;         // gate: the sun cosine changes sign along a surface segment -> plain path
};
// Pixels the surrogate composite hands to the plain integrator: entry =
// kind << 30 | (y * width + x).  count and next are reset by each frame.
enum : uint32_t { kQueueSurface = 0u, kQueueSurfaceCheck = 1u, kQueueSkyCheck = 2u };
struct SurrogateQueue {
  uint32_t* items;    // capacity = width * height
  uint32_t* count;    // [0] = entries, [1] = fallback ticket
  uint32_t* status;   // bit 0 set when a block's tensor-core MMA timed out;
                      // kept across frames until the owner reads and clears it
  float* stats;       // null or kSurrogateStats floats, accumulated
  float check_fraction;
  uint32_t seed;
  // Calibration of the aerial network from the checked pixels (null lm: off).
  // lm: width x height x 3 floats in storage order (the image's contiguous
  // axis first): each MLP surface pixel's network in-scattering, x < 0 where
  // none is to be rescaled.  tiles: per calibration tile (side 1 <<
  // tile_shift, tiles_x per row) the checked pixels' summed log ratios
  // (RGB) and their count.
  float* lm;
  float* tiles;
  int tile_shift, tiles_x;
  // The sky-pixel workload's calibration marks its network pixels here
  // instead (one byte per pixel in storage order; the output image holds
  // the network radiance itself).  Null: not that workload.
  uint8_t* net_mask;
};
// a calibration tile applies when it holds this many checked pixels; each
// checked pixel's log ratio is clamped to +-kCalibrationClamp
constexpr int kCalibrationMinChecks = 4;
constexpr float kCalibrationClamp = 0.3f;
// stats: checked pixels, sum of their relative errors, max relative error,
// gated surface pixels (plain integrator), MLP surface pixels, MLP sky
// pixels, gated sky pixels (sky-view LUT), 128-pixel tiles whose tensor-core
// MMA timed out (their MLP pixels took the plain path; 0 unless the hardware
// misbehaves or the wait bound is set to zero)
constexpr int kSurrogateStats = 8;
struct SampleShaping {
  float top_fraction;      // share of aerial segments starting at the shell top
  float surface_fraction;  // share ending at an altitude in [surface_min, surface_max]
  float surface_min, surface_max;
  float x0_lo, x0_hi;      // feature 0 (start altitude) drawn uniform in [x0_lo, x0_hi] when x0_lo < x0_hi
  float sun_angle_fraction;  // share whose sun zenith at the start is uniform in angle in [0, sun_angle_max]
  float sun_angle_max;       // radians
};
cudaError_t launch_gen_samples(const SurrogateSetDev* sets, int n_sets, int kind, long long n, unsigned long long seed,
                               const SampleShaping& shaping, const float E[3], float ar, float* features,
                               float* targets, unsigned long long* counter, cudaStream_t s);
size_t surrogate_smem_bytes(const SurrogateNets& nets);
// Sky radiance of every pixel: mode 0 the plain integrator per pixel, 1 the
// sky network (plain where a gate trips; status bit 0 set on a tensor-core
// timeout), 2 the sky-view LUT.
cudaError_t launch_sky_pixels(int mode, const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                              const float4* tlut, const float4* mslut, const float4* svlut, const SurrogateNets& nets,
                              uint32_t* status, float* out, unsigned long long* counter, int sm_count, cudaStream_t s,
                              const SurrogateQueue* calibration = nullptr);
cudaError_t launch_composite_surrogate(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                                       const float* scene, const float* space, const int32_t* sid, const float* pos,
                                       const float4* tlut, const float4* mslut, const float4* svlut,
                                       const SurrogateNets& nets, const SurrogateQueue& Q, float* hdr,
                                       unsigned long long* counter, int sm_count, cudaStream_t s,
                                       const struct ShadeParams* shade = nullptr,
                                       const struct ShadeImages* shade_images = nullptr);

// atm_composite_noalloc: the per-device address of the file-scope tile
// scratch (looked up on the first call on each device), its capacity in
// 16x16 tiles, and the COMPOSITE-view launch that uses it.
constexpr int kMaxDevices = 64;
int noalloc_max_tiles();
cudaError_t noalloc_tile_scratch(uint32_t** out, cudaStream_t s);
cudaError_t launch_composite_noalloc(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                                     const float* scene, const float* space, const int32_t* sid, const float* pos,
                                     const float4* tlut, const float4* mslut, const float4* svlut, float* hdr,
                                     uint32_t* tile_scratch, unsigned long long* samples_out, cudaStream_t s);

// Display post-process (atm_post.cu), float32 constants rounded on the host
// the way the reference's Taichi trace rounds them.
struct PostParams {
  int hw, hh;             // bloom planes: max((W + 1) / 2, 1) x max((H + 1) / 2, 1) float4 texels
  int x_fast;             // image and bloom planes with x the contiguous axis ([y][x]); else [x][y]
  float threshold, knee;  // f32(bloom_threshold), f32(bloom_knee)
  float two_knee;         // f32(2 knee)
  float knee_div;         // f32(max(4 knee, 1e-6))
  float clamp;            // f32(bloom_clamp)
};
// Extract into bloom_a, `passes` blur passes ping-ponging between the planes
// (*bloom_out: the plane holding the result), resolve into display.
cudaError_t launch_post(const PostParams& Q, const ImageLayout& L, const float* hdr, float* display, float4* bloom_a,
                        float4* bloom_b, float exposure, float strength, int passes, bool use_bloom, bool tone_map,
                        const float4** bloom_out, cudaStream_t s);
// Surface shading (atm_shade.cu): the kernel's float32 arguments and the
// quantities the reference forms from them once per frame, rounded on the host.
struct ShadeParams {
  float sun[3], E[3], right[3], up[3], fwd[3];  // global frame
  int advanced;                                 // advanced ocean BRDF on
  float roughness, f0, sky_strength;
  float extinction[3];         // f32(absorption) + f32(scattering)
  float scattering_albedo[3];  // scattering / max(extinction, 1e-6)
  float max_depth, eta;        // eta = 1 / f32(refraction_index)
  float strength, max_offset;  // refraction strength, max offset (pixels)
  float solar_slope_variance;  // tanf(f32(sun angular radius))^2
  float tanfov;
  float four_pi;               // f32(4 pi)
  int mode;                    // 0 lit, otherwise albedo
  int32_t ocean_id;            // surface id of ocean pixels
};
// Images of one call: float images with the layout's channels per element,
// scalar and id images with one value per element, all at the same element
// strides.
struct ShadeImages {
  const float* position;
  const float* normal;
  const float* albedo;
  const float* water_depth;
  const float* seabed_albedo;
  const float* seabed_normal;
  const float* slope_variance;
  const int32_t* surface_id;
  const float* terrain_position;
  const float* terrain_normal;
  const float* terrain_albedo;
  const int32_t* terrain_surface_id;
  const float* sun_transmittance;
  const float* sky_radiance;
  float* surface_hdr;
};
cudaError_t launch_shade_surface(const ShadeParams& S, const ImageLayout& L, const ShadeImages& I, cudaStream_t s);
// The fused frame: surface lighting, shading and the COMPOSITE view per pixel
// (I.sun_transmittance, I.sky_radiance and I.surface_hdr are not used).
cudaError_t launch_frame(const DevParams& P, const ImageLayout& L, const CompositeScalars& A, const ShadeParams& S,
                         const ShadeImages& I, const float* space, const float4* tlut, const float4* mslut,
                         const float4* svlut, float* hdr, unsigned long long* sample_counter, cudaStream_t s);

// ---- terrain raster (the G-buffer producer) --------------------------------
// One emitted (clipped) triangle: vertex view positions, normals, material
// weights, heights and cell ids, its screen setup (pixels snapped to 1/256,
// view depth), edge equations, top-left flags (bit k: edge k) and source id.
// The setup the depth passes read comes first, 80 bytes; the attributes the
// resolve reads for the winning triangle follow.  240 bytes, 16-byte
// aligned: written and read as float4.
struct alignas(16) RasterSetup {
  float screen[3][3];
  float eq[3][3];
  float inv_area;
  int32_t tl;
};
struct alignas(16) RasterTri {
  RasterSetup s;
  float v[3][3], n[3][3], m[3][4], h[3];
  int32_t c[3];
  int32_t src;
  int32_t pad[3];
};
static_assert(sizeof(RasterSetup) == 80 && sizeof(RasterTri) == 240, "raster record layout");
struct RasterStream {
  RasterTri* tris;
  uint32_t* count;  // [0] triangles emitted (may exceed capacity: only capacity are stored),
                    // [1] large triangles listed, [2..3] the 64-bit work ticket of their blocks
  long long capacity;
  uint32_t* large;                 // capacity: the emitted triangles too large for one warp
  uint32_t* large_tiles;           // capacity: their pixel-tile counts
  unsigned long long* tile_prefix; // capacity + 1: exclusive prefix of the tile counts
  unsigned long long* block_sums;  // kRasterScanBlocks + 1: the prefix's per-block partial sums
};
constexpr int kRasterScanBlocks = 256;
struct RasterMeshDev {
  const float* view;       // [patches][vertices][3]
  const float* normal;     // [patches][vertices][3]
  const float* material;   // [patches][vertices][4]
  const float* height;     // [patches][vertices]
  const int32_t* cell;     // [patches][vertices]
  const int32_t* triangles;  // [triangles_per_patch][3]
  const int32_t* active;     // [n_active] slots
  const int32_t* skirt_mask; // [patches] or null
  const int32_t* slot_level; // [patches] or null (view mode 2)
  int patches, vertices_per_patch, triangles_per_patch, surface_triangles_per_patch, resolution, n_active;
};
// G-buffer outputs at the layout's element strides: position, normal and
// albedo with L.channels floats per element, material 4 floats, depth and
// height one float, ids one int32.
struct RasterOutDev {
  float* depth;
  float* position;
  float* normal;
  float* albedo;
  float* material;
  float* height;
  int32_t* surface_id;
  int32_t* cell_id;
  float* t_position;  // the terrain snapshot (null t_surface_id: not written)
  float* t_normal;
  float* t_albedo;
  int32_t* t_surface_id;
};
cudaError_t launch_raster(const RasterMeshDev& M, const RasterStream& S, const ImageLayout& L,
                          unsigned long long* depth_key, const RasterOutDev& O, float near, float tf, int mode,
                          int sm_count, cudaStream_t s);

// ---- ocean coverage (the sea-level part of the G-buffer) --------------------
constexpr int kOceanCascades = 3;
constexpr int32_t kOceanSurfaceId = 2147000000;  // OCEAN_SURFACE_ID
// The per-frame wave spectrum: kOceanCascades x n x n texels indexed
// [cascade][x][y] (x along the cascade's u axis): (height, dh/du, dh/dv, 0),
// the horizontal displacement and its 2x2 Jacobian (row-major).
struct OceanSpectrum {
  float4* height_gradient;
  float2* displacement;
  float4* jacobian;
  int n;
};
// One frame's scalars, rounded to float32 as the reference's kernel arguments.
struct OceanFrame {
  float radius, altitude, tf, wind, max_displacement, geometry_max_distance, normal_strength, max_visible_depth;
  float east[3], up[3], north[3], right[3], vup[3], fwd[3], albedo[3];
  float offsets[kOceanCascades][2];
  float variances[kOceanCascades];
  int geometry_cascades, enabled, debug_mode;
};
// The G-buffer images it reads and overwrites, at the layout's element
// strides: position, normal, albedo, seabed albedo and normal with
// L.channels floats, material 4 floats, the rest one value.
struct OceanImages {
  float* depth;
  float* position;
  float* normal;
  float* albedo;
  float* material;
  float* height;
  float* water_depth;
  float* seabed_albedo;
  float* seabed_normal;
  float* slope_variance;
  int32_t* surface_id;
  int32_t* cell_id;
};
cudaError_t launch_ocean_spectrum(const OceanSpectrum& S, float time_s, float amplitude_scale, float choppiness,
                                  cudaStream_t s);
cudaError_t launch_ocean_coverage(const OceanSpectrum& S, const OceanFrame& F, const ImageLayout& L,
                                  const OceanImages& G, cudaStream_t s);

// Whether x is the image's contiguous axis (the orientation of its bloom planes).
bool image_x_fast(const ImageLayout& L);
// A bloom plane of orientation Q.x_fast copied into dst as float4 [y][x].
cudaError_t launch_post_read_bloom(const PostParams& Q, const float4* bloom, float4* dst, cudaStream_t s);

}  // namespace atm
