// atm_batch.cu - many sky-view and aerial-perspective LUTs in one persistent
// launch (time snapshots x cameras x parameter sets, uneven LUT sizes).
//
// The reference builds one LUT per kernel launch (atmosphere/renderer.py
// :1208, :1304).  Here a job table describes every LUT of a batch; each job is
// split into work items of `per_item` texels (sky-view) or froxel columns
// (aerial).  A grid of blocks_per_sm x SM-count blocks stays resident; each
// warp takes the next work item from an atomic ticket, finds its job by
// binary search over the item prefix sums, copies the job's parameters into
// its shared-memory slot and evaluates the texels/columns with the same
// warp-level functions as the single-LUT kernels.  Warps never wait on each
// other (the ticket is a plain atomicAdd), so uneven job sizes balance
// without barriers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "atm_capi.h"
#include "atm_device.cuh"
#include "atm_kernels.h"
#include "atm_lut_warp.cuh"

namespace atm {

struct BatchJobDev {
  DevParams P;  // the job's parameter set with its own LUT size
  float4* out;
  const float4* tlut;
  const float4* mslut;
  int kind;      // ATM_LUT_SKY_VIEW or ATM_LUT_AERIAL
  int units;     // texels (sky-view) or columns (aerial)
  int per_item;  // units per work item
  float bottom, cam_alt, sun_cos, ar, aspect, tanfov;
  f3 sun, E, right, up, fwd;
};

namespace {

constexpr int kBatchWarps = 8;  // 256-thread blocks

__global__ void __launch_bounds__(256, 3) k_batch(const BatchJobDev* __restrict__ jobs,
                                               const long long* __restrict__ prefix, int n_jobs, long long n_items,
                                               unsigned long long* __restrict__ ticket,
                                               unsigned long long* __restrict__ samples_counter) {
  __shared__ DevParams s_params[kBatchWarps];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  uint32_t samples = 0;
  int loaded = -1;
  for (;;) {
    unsigned long long item = 0;
    if (lane == 0) item = atomicAdd(ticket, 1ull);
    item = __shfl_sync(kFull, item, 0);
    if (item >= static_cast<unsigned long long>(n_items)) break;
    // job j: prefix[j] <= item < prefix[j + 1]
    int lo = 0, hi = n_jobs;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (prefix[mid] <= static_cast<long long>(item)) lo = mid;
      else hi = mid;
    }
    const BatchJobDev* J = jobs + lo;
    if (lo != loaded) {  // stage the job's parameters in this warp's slot
      __syncwarp();
      const int* src = reinterpret_cast<const int*>(&J->P);
      int* dst = reinterpret_cast<int*>(&s_params[warp]);
      for (int k = lane; k < int(sizeof(DevParams) / sizeof(int)); k += 32) dst[k] = src[k];
      __syncwarp();
      loaded = lo;
    }
    const DevParams& P = s_params[warp];
    const long long local = static_cast<long long>(item) - prefix[lo];
    const int per = J->per_item;
    const int u0 = static_cast<int>(local * per);
    const int u1 = min(u0 + per, J->units);
    if (J->kind == ATM_LUT_SKY_VIEW) {
      const float sc = J->sun_cos;
      const float ss = sqrtf(mx(1.0f - sc * sc, 0.0f));
      const Frame F = make_frame(P, J->tlut, J->mslut, J->bottom, J->ar, mk(ss, sc, 0.0f), J->E);
      for (int u = u0; u < u1; ++u) samples += sky_view_texel(P, F, J->cam_alt, u % P.sv_w, u / P.sv_w, J->out);
    } else {
      const Frame F = make_frame(P, J->tlut, J->mslut, J->bottom, J->ar, J->sun, J->E);
      const AerialView V{J->aspect, J->cam_alt, J->right, J->up, J->fwd, J->tanfov};
      for (int u = u0; u < u1; ++u) samples += aerial_column(P, F, V, u % P.ap_w, u / P.ap_w, J->out);
    }
  }
  warp_count(samples, samples_counter);
}

}  // namespace

cudaError_t launch_batch(const BatchJobDev* jobs, const long long* prefix, int n_jobs, long long n_items,
                         unsigned long long* ticket, unsigned long long* samples, int blocks, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  k_batch<<<blocks, 256, 0, s>>>(jobs, prefix, n_jobs, n_items, ticket, samples);
  return cudaGetLastError();
}

size_t batch_job_size() { return sizeof(BatchJobDev); }

// Fill one device job descriptor from the ABI job (host side).
void fill_batch_job(BatchJobDev& d, const DevParams& set_params, const AtmBatchJob& j, float4* arena,
                    const float4* tlut, const float4* mslut, double radius, const double E[3], double ar_rad,
                    int per_item) {
  std::memset(&d, 0, sizeof(d));
  d.P = set_params;
  d.kind = j.kind;
  d.out = arena + j.output_offset;
  d.tlut = tlut;
  d.mslut = mslut;
  d.bottom = float(radius);
  d.cam_alt = float(j.camera_altitude_m);
  d.ar = float(ar_rad);
  d.E = {float(E[0]), float(E[1]), float(E[2])};
  d.per_item = per_item;
  if (j.kind == ATM_LUT_SKY_VIEW) {
    d.P.sv_w = j.width;
    d.P.sv_h = j.height;
    d.units = j.width * j.height;
    d.sun_cos = float(j.sun_zenith_cosine);
  } else {
    d.P.ap_w = j.width;
    d.P.ap_h = j.height;
    d.P.ap_d = j.depth;
    d.units = j.width * j.height;
    d.sun = {float(j.sun_local[0]), float(j.sun_local[1]), float(j.sun_local[2])};
    d.right = {float(j.view_basis[0]), float(j.view_basis[1]), float(j.view_basis[2])};
    d.up = {float(j.view_basis[3]), float(j.view_basis[4]), float(j.view_basis[5])};
    d.fwd = {float(j.view_basis[6]), float(j.view_basis[7]), float(j.view_basis[8])};
    d.tanfov = float(j.tangent_half_fov);
    d.aspect = float(j.frame_width) / float(j.frame_height);
  }
}

}  // namespace atm
