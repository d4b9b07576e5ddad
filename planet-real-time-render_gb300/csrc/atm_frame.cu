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
#include "atm_frame_paths.cuh"
#include "atm_kernels.h"

namespace atm {
namespace {

constexpr unsigned kFull = 0xffffffffu;

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
  if (sid[e] >= 0) surface_lighting(P, F, cam_alt, right, up, fwd, ld3(pos + o), st, sky);
  out_t[o + 0] = st.x;
  out_t[o + 1] = st.y;
  out_t[o + 2] = st.z;
  out_sky[o + 0] = sky.x;
  out_sky[o + 1] = sky.y;
  out_sky[o + 2] = sky.z;
}

// One pixel of the COMPOSITE view (:1860-1940) given its surface colour
// (scene_hdr) and surface id: writes hdr and adds the pixel's radiance
// samples to `samples`.  Shared by the composite, its no-allocation variant
// and the fused frame so that they cannot drift apart.
__device__ __forceinline__ void composite_pixel_with(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                                                     const Frame& F, f3 color, int32_t sidv,
                                                     const float* __restrict__ space, const float* __restrict__ pos,
                                                     const float4* __restrict__ svlut, float* __restrict__ hdr, int x,
                                                     int y, uint32_t& samples) {
  const size_t o = pix_offset(L, x, y) * L.channels;
  PixelRay pr = pixel_ray(L, A, x, y);
  if (sidv >= 0) {
    const RayGeom G = camera_ray_geom(P, A.bottom, A.cam_alt, pr.ray);
    float sd = norm(ld3(pos + o));
    float start, end;
    if (surface_interval(P, G, A.bottom, sd, start, end)) {
      f3 scat = integrate_surface(P, F, G, pr.ray, start, end, samples);
      f3 tr = surface_segment_t(P, F, G, pr.ray, start, end);
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
__device__ __forceinline__ void composite_pixel(const DevParams& P, const ImageLayout& L, const CompositeScalars& A,
                                                const float* __restrict__ scene, const float* __restrict__ space,
                                                const int32_t* __restrict__ sid, const float* __restrict__ pos,
                                                const float4* __restrict__ tlut, const float4* __restrict__ mslut,
                                                const float4* __restrict__ svlut, float* __restrict__ hdr, int x,
                                                int y, uint32_t& samples) {
  const size_t e = pix_offset(L, x, y);
  const Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
  composite_pixel_with(P, L, A, F, ld3(scene + e * L.channels), sid[e], space, pos, svlut, hdr, x, y, samples);
}

// COMPOSITE view (:1860-1940): the per-frame path.
__global__ void __launch_bounds__(256, 3) k_composite(DevParams P, ImageLayout L, CompositeScalars A,
                                                   const float* __restrict__ scene, const float* __restrict__ space,
                                                   const int32_t* __restrict__ sid, const float* __restrict__ pos,
                                                   const float4* __restrict__ tlut, const float4* __restrict__ mslut,
                                                   const float4* __restrict__ svlut, float* __restrict__ hdr,
                                                   unsigned long long* counter) {
  int x, y;
  uint32_t samples = 0;
  if (tile_pixel(L, x, y)) composite_pixel(P, L, A, scene, space, sid, pos, tlut, mslut, svlut, hdr, x, y, samples);
  warp_count(samples, counter);
}

// The frame in one pass: per pixel the surface lighting (:1422-1472), the
// surface shading (renderer.py:1277-1575) and the COMPOSITE view
// (:1860-1940), with the lighting and the shaded colour in registers instead
// of the three full-resolution images that the separate calls write and
// read back.
__global__ void __launch_bounds__(256, 3) k_frame(DevParams P, ImageLayout L, CompositeScalars A, ShadeParams S,
                                               ShadeImages I, const float* __restrict__ space,
                                               const float4* __restrict__ tlut, const float4* __restrict__ mslut,
                                               const float4* __restrict__ svlut, float* __restrict__ hdr,
                                               unsigned long long* counter) {
  int x, y;
  uint32_t samples = 0;
  if (tile_pixel(L, x, y)) {
    const size_t e = pix_offset(L, x, y);
    const int32_t sidv = I.surface_id[e];
    const Frame F = make_frame(P, tlut, mslut, A.bottom, A.ar, arr3(A.sun), arr3(A.E));
    const f3 scene = shaded_scene(P, F, A, S, L, I, x, y, e, sidv);
    composite_pixel_with(P, L, A, F, scene, sidv, space, I.position, svlut, hdr, x, y, samples);
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
    const RayGeom G = camera_ray_geom(P, A.bottom, A.cam_alt, pr.ray);
    const bool surface = sid[e] >= 0;
    f3 color = ld3(scene + o);
    switch (A.view) {
      case ATM_VIEW_SKY_VIEW:
        color = sample_sky_view(P, svlut, pr.ray, F.sun, A.sky_alt, A.bottom);
        break;
      case ATM_VIEW_CAMERA_TRANSMITTANCE:
        color = camera_t(P, F, G, pr.ray);
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
        if (surface && surface_interval(P, G, A.bottom, norm(ld3(pos + o)), start, end))
          color = integrate_surface(P, F, G, pr.ray, start, end, samples);
        break;
      }
      case ATM_VIEW_AERIAL_FROXEL_ONLY: {
        color = splat(0.0f);
        if (surface) {
          float s, e2;
          bool valid;
          aerial_prefix_of(P, G, A.bottom, s, e2, valid);
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
          if (surface_interval(P, G, A.bottom, norm(ld3(pos + o)), start, end))
            color = surface_segment_t(P, F, G, pr.ray, start, end);
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

cudaError_t launch_frame(const DevParams& P, const ImageLayout& L, const CompositeScalars& A, const ShadeParams& S,
                         const ShadeImages& I, const float* space, const float4* tlut, const float4* mslut,
                         const float4* svlut, float* hdr, unsigned long long* sample_counter, cudaStream_t s) {
  k_frame<<<tile_grid(L), 256, 0, s>>>(P, L, A, S, I, space, tlut, mslut, svlut, hdr, sample_counter);
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

// COMPOSITE view of k_composite (the same composite_pixel); the block's
// sample count goes to its tile slot instead of an atomic counter (every
// launched block writes its slot).
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
  uint32_t samples = 0;
  if (tile_pixel(L, x, y)) composite_pixel(P, L, A, scene, space, sid, pos, tlut, mslut, svlut, hdr, x, y, samples);
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

// The array's device address on the current device.  Outside a stream
// capture the address is looked up afresh (a device reset reloads the module
// and may move the array); while `s` is capturing, the address of the last
// lookup on this device is used, so the first call on a device must come
// before any capture.
cudaError_t noalloc_tile_scratch(uint32_t** out, cudaStream_t s) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return e;
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  const bool capturing = cudaStreamIsCapturing(s, &capture) != cudaSuccess || capture != cudaStreamCaptureStatusNone;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!capturing) {
    void* address = nullptr;
    e = cudaGetSymbolAddress(&address, g_noalloc_tile_samples);  // with `device` current
    if (e != cudaSuccess) return e;
    g_noalloc_address[device] = static_cast<uint32_t*>(address);
  } else if (g_noalloc_address[device] == nullptr) {
    return cudaErrorStreamCaptureUnsupported;  // first call on this device inside a capture
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
