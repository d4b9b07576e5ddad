// atm_f32.cuh - IEEE float32 vector arithmetic in a written operation order:
// every multiply, add, divide and square root rounds on its own (no FMA
// contraction), so kernels that restate a float32 reference step by step
// produce its bits.  Shared by the terrain raster and the ocean coverage.
#pragma once

#include <cuda_runtime.h>

namespace atm {
namespace f32 {

struct r3 {
  float x, y, z;
};
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fmx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fmn(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ r3 R3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ r3 radd(r3 a, r3 b) { return {add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)}; }
__device__ __forceinline__ r3 rsub(r3 a, r3 b) { return {sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)}; }
__device__ __forceinline__ r3 rscale(r3 a, float s) { return {mul(a.x, s), mul(a.y, s), mul(a.z, s)}; }
__device__ __forceinline__ float rdot(r3 a, r3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
__device__ __forceinline__ r3 rcross(r3 a, r3 b) {
  return {sub(mul(a.y, b.z), mul(a.z, b.y)), sub(mul(a.z, b.x), mul(a.x, b.z)), sub(mul(a.x, b.y), mul(a.y, b.x))};
}
// Taichi's normalized(): (1 / (|v| + 0)) * v
__device__ __forceinline__ r3 rnormalized(r3 v) {
  const float inv = dv(1.0f, add(__fsqrt_rn(rdot(v, v)), 0.0f));
  return {mul(inv, v.x), mul(inv, v.y), mul(inv, v.z)};
}
}  // namespace f32
}  // namespace atm
