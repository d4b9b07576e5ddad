// atm_shade.cu - the surface shading that consumes prepare_frame's surface
// lighting (PlanetRenderer._shade_surface, src/planet_renderer/renderer.py
// :1277-1575) on sm_103a: Lambertian land under the transmitted sun and the
// sky radiance; ocean pixels (advanced ocean on) with a GGX-style sun
// specular, Fresnel sky reflection and a water body over a seabed that is
// reconstructed along the refracted view ray from the opaque terrain
// snapshot (bilinear over four neighbours, depth-tested).
//
// One thread per pixel along the image's contiguous axis; HBM-bound (~200 B
// per ocean pixel, ~90 B per land pixel).  Arithmetic is IEEE float32 in the
// reference's operation order without contraction (__fmul_rn / __fadd_rn),
// so results follow the reference's to the last bits of expf.
#include <cuda_runtime.h>

#include <cstdint>

#include "atm_kernels.h"
#include "atm_shade.cuh"

namespace atm {

namespace {

using namespace shading;

__global__ void __launch_bounds__(256) k_shade_surface(ShadeParams S, ImageLayout L, ShadeImages I) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= int64_t(L.width) * L.height) return;
  int x, y;
  if (L.sy <= L.sx) {  // y contiguous: the reference's (W, H, 3) layout
    x = int(i / L.height);
    y = int(i % L.height);
  } else {
    y = int(i / L.width);
    x = int(i % L.width);
  }
  const int64_t e = int64_t(x) * L.sx + int64_t(y) * L.sy;
  const int c = L.channels;
  const int32_t sid = I.surface_id[e];
  v3 T = V(0.0f, 0.0f, 0.0f), sky = V(0.0f, 0.0f, 0.0f);
  if (sid >= 0 && S.mode == 0) {
    T = ld(I.sun_transmittance, e, c);
    sky = ld(I.sky_radiance, e, c);
  }
  const v3 color = vmax0(shade_pixel(S, L, I, x, y, e, sid, T, sky));
  float* out = I.surface_hdr + e * c;
  out[0] = color.x;
  out[1] = color.y;
  out[2] = color.z;
}

}  // namespace

cudaError_t launch_shade_surface(const ShadeParams& S, const ImageLayout& L, const ShadeImages& I, cudaStream_t s) {
  const int64_t n = int64_t(L.width) * L.height;
  k_shade_surface<<<unsigned((n + 255) / 256), 256, 0, s>>>(S, L, I);
  return cudaGetLastError();
}

}  // namespace atm
