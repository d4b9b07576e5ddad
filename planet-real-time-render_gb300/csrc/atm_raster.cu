// atm_raster.cu - the terrain raster that produces the G-buffer the
// atmosphere stage consumes (PlanetRenderer._clip, _emit,
// _raster_depth_direct, _resolve_raster; src/planet_renderer/renderer.py
// :628-1269) on sm_103a.
//
//  * k_raster_clip: thread per source triangle of the active patches:
//    back-face culling of surface triangles (skirts are double-sided), the
//    clip-code trivial reject, Sutherland-Hodgman clipping against the near
//    plane and the four frustum sides, and the emission (an atomic append)
//    of each resulting triangle with its screen setup: projection snapped to
//    1/256 pixel, edge equations, top-left flags, inverse area;
//  * k_raster_depth (+ k_raster_scan_*, k_raster_depth_tiles): coverage
//    by the edge equations with the top-left rule and a 64-bit atomic
//    minimum of (depth bits << 32 | triangle) per pixel; small triangles by
//    one thread, medium ones by a warp, large ones cut into 8 x 32 pixel
//    tiles spread over the whole grid;
//  * k_raster_resolve: thread per pixel: the winning triangle's
//    perspective-correct position, normal, material weights and height, the
//    dominant vertex's cell id and the albedo of the view mode.
//
// Arithmetic is IEEE float32 in the reference's operation order without
// contraction (__fmul_rn / __fadd_rn / __fdiv_rn), so every written value
// equals the reference's.  Triangles get their stream slot from an atomic
// counter, so their order (the key's low bits) differs from the
// reference's sequential order: only the winner of an exact depth tie can
// differ.
#include <cuda_runtime.h>

#include <cstdint>

#include "atm_f32.cuh"
#include "atm_kernels.h"

namespace atm {

namespace {

using namespace f32;

constexpr int kClipVerts = 8;      // MAX_CLIP_VERTICES
constexpr int kClipTris = 6;       // MAX_CLIPPED_TRIANGLES
constexpr unsigned long long kSentinel = ~0ull;

struct r4 {
  float v[4];
};

// One clip-space vertex with its attributes.
struct CVert {
  r3 p, n;
  r4 m;
  float h;
  int32_t c;
};

__device__ __forceinline__ int clip_code(r3 p, float near, float tx, float ty) {
  int code = 0;
  if (p.z < near) code |= 1;
  if (p.x < mul(-p.z, tx)) code |= 2;
  if (p.x > mul(p.z, tx)) code |= 4;
  if (p.y < mul(-p.z, ty)) code |= 8;
  if (p.y > mul(p.z, ty)) code |= 16;
  return code;
}
__device__ __forceinline__ float clip_distance(r3 p, int plane, float near, float tx, float ty) {
  if (plane == 1) return add(p.x, mul(p.z, tx));
  if (plane == 2) return add(-p.x, mul(p.z, tx));
  if (plane == 3) return add(p.y, mul(p.z, ty));
  if (plane == 4) return add(-p.y, mul(p.z, ty));
  return sub(p.z, near);
}
__device__ __forceinline__ r3 edge_coeff(float ax, float ay, float bx, float by) {
  return {sub(ay, by), sub(bx, ax), sub(mul(sub(by, ay), ax), mul(sub(bx, ax), ay))};
}
__device__ __forceinline__ int top_left(float ax, float ay, float bx, float by, float o) {
  const float dx = mul(sub(bx, ax), o), dy = mul(sub(by, ay), o);
  return (dy > 0.0f) || (dy == 0.0f && dx < 0.0f);
}

union TriBits {
  RasterTri t;
  float4 v[sizeof(RasterTri) / 16];
};
union SetupBits {
  RasterSetup s;
  float4 v[sizeof(RasterSetup) / 16];
};
__device__ __forceinline__ RasterSetup load_setup(const RasterTri* t) {
  SetupBits u;
  const float4* p = reinterpret_cast<const float4*>(t);
#pragma unroll
  for (int k = 0; k < int(sizeof(RasterSetup) / 16); ++k) u.v[k] = p[k];
  return u.s;
}

// _emit :628-686: the record is assembled in registers and stored as float4s
__device__ void emit(const RasterMeshDev& M, RasterStream S, int32_t src, const CVert (&v)[3], float tf,
                     float aspect, int width, int height) {
  const uint32_t s = atomicAdd(S.count, 1u);
  if (s >= uint32_t(S.capacity)) return;  // counted, not stored (the reference's s >= capacity)
  TriBits u;
  RasterTri& T = u.t;
  float sp[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const r3 p = v[k].p;
    T.v[k][0] = p.x;
    T.v[k][1] = p.y;
    T.v[k][2] = p.z;
    T.n[k][0] = v[k].n.x;
    T.n[k][1] = v[k].n.y;
    T.n[k][2] = v[k].n.z;
#pragma unroll
    for (int i = 0; i < 4; ++i) T.m[k][i] = v[k].m.v[i];
    T.h[k] = v[k].h;
    T.c[k] = v[k].c;
    float px = mul(add(mul(dv(p.x, mul(mul(p.z, tf), aspect)), 0.5f), 0.5f), float(width));
    float py = mul(add(mul(dv(p.y, mul(p.z, tf)), 0.5f), 0.5f), float(height));
    px = dv(floorf(add(mul(px, 256.0f), 0.5f)), 256.0f);
    py = dv(floorf(add(mul(py, 256.0f), 0.5f)), 256.0f);
    sp[k][0] = px;
    sp[k][1] = py;
    sp[k][2] = p.z;
    T.s.screen[k][0] = px;
    T.s.screen[k][1] = py;
    T.s.screen[k][2] = p.z;
  }
  const float ax = sp[0][0], ay = sp[0][1], bx = sp[1][0], by = sp[1][1], cx = sp[2][0], cy = sp[2][1];
  const float area = sub(mul(sub(bx, ax), sub(cy, ay)), mul(sub(by, ay), sub(cx, ax)));  // _edge(a, b, c)
  const float abs_area = fabsf(area);
  const float sg = area > 0.0f ? 1.0f : -1.0f;
  T.s.inv_area = abs_area > 1e-8f ? dv(1.0f, abs_area) : 0.0f;
  const r3 e0 = rscale(edge_coeff(bx, by, cx, cy), sg);
  const r3 e1 = rscale(edge_coeff(cx, cy, ax, ay), sg);
  const r3 e2 = rscale(edge_coeff(ax, ay, bx, by), sg);
  T.s.eq[0][0] = e0.x, T.s.eq[0][1] = e0.y, T.s.eq[0][2] = e0.z;
  T.s.eq[1][0] = e1.x, T.s.eq[1][1] = e1.y, T.s.eq[1][2] = e1.z;
  T.s.eq[2][0] = e2.x, T.s.eq[2][1] = e2.y, T.s.eq[2][2] = e2.z;
  T.s.tl =
      top_left(bx, by, cx, cy, sg) | (top_left(cx, cy, ax, ay, sg) << 1) | (top_left(ax, ay, bx, by, sg) << 2);
  T.src = src;
  T.pad[0] = T.pad[1] = T.pad[2] = 0;
  float4* dst = reinterpret_cast<float4*>(S.tris + s);
#pragma unroll
  for (int k = 0; k < int(sizeof(RasterTri) / 16); ++k) dst[k] = u.v[k];
}

// _clip :731-901
__global__ void __launch_bounds__(128) k_raster_clip(RasterMeshDev M, RasterStream S, float near, float tf,
                                                     int width, int height) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int ltc = M.triangles_per_patch;
  if (i >= (long long)M.n_active * ltc) return;
  const float aspect = dv(float(width), float(height));
  const float tx = mul(tf, aspect), ty = tf;
  const int slot = M.active[i / ltc];
  if (slot < 0 || slot >= M.patches) return;  // not a patch: nothing to draw
  const int local_id = int(i % ltc);
  const int32_t source_id = slot * ltc + local_id;
  const int stc = M.surface_triangles_per_patch;
  if (local_id >= stc) {  // a skirt: enabled per patch edge
    const int edge = (local_id - stc) / (M.resolution * 2);
    if (M.skirt_mask == nullptr || (M.skirt_mask[slot] & (1 << edge)) == 0) return;
  }
  const int32_t* ids = M.triangles + 3 * local_id;
  for (int k = 0; k < 3; ++k)
    if (ids[k] < 0 || ids[k] >= M.vertices_per_patch) return;  // a vertex outside the patch: dropped
  // positions first: culled and rejected triangles read nothing else
  CVert v[3];
  long long ev[3];
  for (int k = 0; k < 3; ++k) {
    const long long e = (long long)slot * M.vertices_per_patch + ids[k];
    ev[k] = e;
    v[k].p = R3(M.view[3 * e], M.view[3 * e + 1], M.view[3 * e + 2]);
  }
  // ordinary terrain back faces are culled; skirts stay double-sided
  if (local_id < stc) {
    const r3 p0 = v[0].p;
    if (!(rdot(rcross(rsub(v[1].p, p0), rsub(v[2].p, p0)), R3(-p0.x, -p0.y, -p0.z)) < 0.0f)) return;
  }
  const int c0 = clip_code(v[0].p, near, tx, ty), c1 = clip_code(v[1].p, near, tx, ty),
            c2 = clip_code(v[2].p, near, tx, ty);
  if (c0 & c1 & c2) return;  // all three outside one plane
  for (int k = 0; k < 3; ++k) {
    const long long e = ev[k];
    v[k].n = R3(M.normal[3 * e], M.normal[3 * e + 1], M.normal[3 * e + 2]);
    for (int j = 0; j < 4; ++j) v[k].m.v[j] = M.material[4 * e + j];
    v[k].h = M.height[e];
    v[k].c = M.cell[e];
  }
  if ((c0 | c1 | c2) == 0) {
    emit(M, S, source_id, v, tf, aspect, width, height);
    return;
  }
  // Sutherland-Hodgman over the five planes, ping-ponging two vertex buffers
  CVert buf[2][kClipVerts];
  for (int k = 0; k < 3; ++k) buf[0][k] = v[k];
  int count = 3, rd = 0;
  for (int plane = 0; plane < 5; ++plane) {
    const int wr = 1 - rd;
    int oc = 0;
    for (int vertex = 0; vertex < kClipVerts; ++vertex) {
      if (vertex >= count) break;
      const int prev = (vertex + count - 1) % count;
      const CVert& cur = buf[rd][vertex];
      const CVert& pre = buf[rd][prev];
      const float cd = clip_distance(cur.p, plane, near, tx, ty);
      const float pd = clip_distance(pre.p, plane, near, tx, ty);
      const bool ci = cd >= 0.0f, pi = pd >= 0.0f;
      if (ci != pi && oc < kClipVerts) {
        const float den = sub(pd, cd);
        const float t = fabsf(den) > 1e-20f ? dv(pd, den) : 0.0f;
        CVert& o = buf[wr][oc];
        o.p = radd(pre.p, rscale(rsub(cur.p, pre.p), t));
        o.n = rnormalized(radd(pre.n, rscale(rsub(cur.n, pre.n), t)));
        for (int j = 0; j < 4; ++j) o.m.v[j] = add(pre.m.v[j], mul(sub(cur.m.v[j], pre.m.v[j]), t));
        o.h = add(pre.h, mul(sub(cur.h, pre.h), t));
        o.c = ci ? cur.c : pre.c;
        ++oc;
      }
      if (ci && oc < kClipVerts) buf[wr][oc++] = cur;
    }
    count = oc;
    rd = wr;
  }
  for (int tri = 0; tri < kClipTris; ++tri) {
    if (tri >= count - 2) break;
    const CVert t3[3] = {buf[rd][0], buf[rd][tri + 1], buf[rd][tri + 2]};
    emit(M, S, source_id, t3, tf, aspect, width, height);
  }
}

__device__ __forceinline__ r3 edge_values(const RasterSetup& T, float px, float py) {
  return {add(add(mul(T.eq[0][0], px), mul(T.eq[0][1], py)), T.eq[0][2]),
          add(add(mul(T.eq[1][0], px), mul(T.eq[1][1], py)), T.eq[1][2]),
          add(add(mul(T.eq[2][0], px), mul(T.eq[2][1], py)), T.eq[2][2])};
}
__device__ __forceinline__ bool inside_edges(const RasterSetup& T, r3 e) {
  return (e.x > 0.0f || (e.x == 0.0f && (T.tl & 1))) && (e.y > 0.0f || (e.y == 0.0f && (T.tl & 2))) &&
         (e.z > 0.0f || (e.z == 0.0f && (T.tl & 4)));
}

// _raster_depth_direct :1158-1206, in three sizes of work.  Each covered
// pixel centre (edge equations with the top-left rule) takes the atomic
// minimum of (depth bits << 32 | triangle); the order of the atomics changes
// no result.  Pixels are walked along y, the depth keys' contiguous axis.
__device__ __forceinline__ void depth_pixel(const RasterSetup& T, int x, int y, int H,
                                            unsigned long long* __restrict__ depth_key, unsigned long long q) {
  const r3 e = edge_values(T, add(float(x), 0.5f), add(float(y), 0.5f));
  if (!inside_edges(T, e)) return;
  const r3 l = rscale(e, T.inv_area);
  const float z = dv(1.0f, fmx(add(add(dv(l.x, T.screen[0][2]), dv(l.y, T.screen[1][2])), dv(l.z, T.screen[2][2])),
                               1e-20f));
  atomicMin(depth_key + (size_t(x) * H + y), ((unsigned long long)__float_as_uint(z) << 32) | q);
}
struct Box {
  int x0, x1, y0, y1;
};
__device__ __forceinline__ Box bbox(const RasterSetup& T, const ImageLayout& L) {
  const float ax = T.screen[0][0], bx = T.screen[1][0], cx = T.screen[2][0];
  const float ay = T.screen[0][1], by = T.screen[1][1], cy = T.screen[2][1];
  return {max(int(floorf(fmn(fmn(ax, bx), cx))), 0), min(int(ceilf(fmx(fmx(ax, bx), cx))), L.width - 1),
          max(int(floorf(fmn(fmn(ay, by), cy))), 0), min(int(ceilf(fmx(fmx(ay, by), cy))), L.height - 1)};
}
constexpr long long kRasterThreadArea = 16;  // bounding boxes up to this many pixels: one thread
constexpr long long kRasterWarpArea = 256;   // up to this: one warp; larger: tiles over the whole grid
constexpr int kRasterTileW = 256, kRasterTileH = 32;  // a large triangle's work item: 256 columns x 32 rows
constexpr int kRasterItemsPerTicket = 4;              // work items a warp takes per ticket

// Whether the edge equations reject a whole tile of pixel centres: an edge
// whose value is negative at the tile's corner where it is largest.  The
// float32 edge value is monotone in x (y) for a non-negative x (y)
// coefficient, so that corner is the tile's largest value as the pixel test
// evaluates it: a rejected tile holds no covered pixel.
__device__ __forceinline__ bool tile_outside(const RasterSetup& T, int xs, int xe, int ys, int ye) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float px = add(float(T.eq[k][0] >= 0.0f ? xe : xs), 0.5f);
    const float py = add(float(T.eq[k][1] >= 0.0f ? ye : ys), 0.5f);
    if (add(add(mul(T.eq[k][0], px), mul(T.eq[k][1], py)), T.eq[k][2]) < 0.0f) return true;
  }
  return false;
}

// A row's conservative span of columns inside the triangle (within
// [xs, xe]), from each edge's crossing: the exact per-pixel test decides,
// the span only bounds the walk.  The crossing is widened by one pixel plus
// a bound on the float32 rounding of the edge value, (|A x| + |B y| + |C|)
// 2^-20 / |A| pixels: every pixel the exact test covers lies inside the
// span.  n = 0: the row holds no covered pixel.
__device__ __forceinline__ void row_span(const RasterSetup& T, float py, int xs, int xe, int& l, int& n) {
  float lo = float(xs), hi = float(xe);
  const float xmag = fmaxf(fabsf(float(xs)), fabsf(float(xe))) + 1.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float A = T.eq[k][0];
    const float By = mul(T.eq[k][1], py);
    const float rest = add(By, T.eq[k][2]);
    if (A == 0.0f) {
      if (rest < 0.0f) hi = -1.0f;  // e = (0 + B y) + C = rest exactly, for every pixel of the row
    } else {
      const float cross = sub(dv(-rest, A), 0.5f);  // pixel index where e crosses 0
      const float margin =
          1.0f + (fabsf(A) * xmag + fabsf(By) + fabsf(T.eq[k][2])) * 9.5367431640625e-07f / fabsf(A);
      if (A > 0.0f)
        lo = fmaxf(lo, floorf(cross - margin));
      else
        hi = fminf(hi, ceilf(cross + margin));
    }
  }
  // NaN crossings compare false and leave the bounds as they were
  lo = fmaxf(lo, float(xs));
  hi = fminf(hi, float(xe));
  l = int(lo);
  n = hi >= lo ? int(hi) - int(lo) + 1 : 0;
}

// One work item of a large triangle, a block of up to 256 columns x 32 rows
// walked by one warp: lane = row computes its span, the spans are prefix-
// summed over the lanes, and the lanes then take the spans' pixels 32 at a
// time (the exact coverage test, the depth and the atomic minimum), so the
// lanes stay busy however thin the triangle.
__device__ __forceinline__ void warp_block(const RasterSetup& T, unsigned long long q, int xs, int xe, int ys, int ye,
                                           int H, unsigned long long* __restrict__ depth_key) {
  const int lane = threadIdx.x & 31;
  const int y = ys + lane;
  int l = 0, n = 0;
  if (y <= ye) row_span(T, add(float(y), 0.5f), xs, xe, l, n);
  int incl = n;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  for (int base = 0; base < total; base += 32) {
    const int i = base + lane;
    int row = 0;  // the first lane whose inclusive count exceeds i
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int probe = __shfl_sync(0xffffffffu, incl, row + step - 1);
      if (probe <= i) row += step;
    }
    const int rl = __shfl_sync(0xffffffffu, l, row), rn = __shfl_sync(0xffffffffu, n, row);
    const int rincl = __shfl_sync(0xffffffffu, incl, row);
    if (i < total) depth_pixel(T, rl + (i - (rincl - rn)), ys + row, H, depth_key, q);
  }
}

// Thread per emitted triangle (grid-stride, warp-aligned): small boxes are
// walked by their own thread, medium ones by the whole warp in turn, large
// ones are listed for k_raster_depth_tiles.
__global__ void __launch_bounds__(256) k_raster_depth(RasterStream S, ImageLayout L,
                                                      unsigned long long* __restrict__ depth_key) {
  const int lane = threadIdx.x & 31;
  const long long n = min((long long)S.count[0], (long long)S.capacity);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
    const long long q = base + lane;
    bool medium = false;
    if (q < n) {
      const RasterSetup T = load_setup(S.tris + q);
      const Box b = bbox(T, L);
      if (T.inv_area > 0.0f && b.x0 <= b.x1 && b.y0 <= b.y1) {
        const long long area = (long long)(b.x1 - b.x0 + 1) * (b.y1 - b.y0 + 1);
        if (area <= kRasterThreadArea) {
          for (int x = b.x0; x <= b.x1; ++x)
            for (int y = b.y0; y <= b.y1; ++y) depth_pixel(T, x, y, L.height, depth_key, (unsigned long long)q);
        } else if (area <= kRasterWarpArea) {
          medium = true;
        } else {
          const uint32_t idx = atomicAdd(S.count + 1, 1u);  // at most one entry per stored triangle
          S.large[idx] = uint32_t(q);
          S.large_tiles[idx] = uint32_t((b.x1 - b.x0 + kRasterTileW) / kRasterTileW) *
                               uint32_t((b.y1 - b.y0 + kRasterTileH) / kRasterTileH);
        }
      }
    }
    unsigned m = __ballot_sync(0xffffffffu, medium);
    while (m) {
      const int leader = __ffs(m) - 1;
      m &= m - 1;
      const long long ql = base + leader;
      const RasterSetup T = load_setup(S.tris + ql);
      const Box b = bbox(T, L);
      const int bh = b.y1 - b.y0 + 1;
      const int area = (b.x1 - b.x0 + 1) * bh;  // at most kRasterWarpArea: 8 pixels per lane
      for (int k = lane; k < area; k += 32)
        depth_pixel(T, b.x0 + k / bh, b.y0 + k % bh, L.height, depth_key, (unsigned long long)ql);
    }
  }
}

// The exclusive prefix of the large triangles' tile counts (64-bit) in three
// launches: per-block sums over kRasterScanBlocks equal ranges, a scan of
// the sums, then each block's own scan offset by its sum's prefix.
__device__ __forceinline__ void scan_range(uint32_t n, uint32_t& lo, uint32_t& hi) {
  const uint32_t per = (n + kRasterScanBlocks - 1) / kRasterScanBlocks;
  lo = min(n, blockIdx.x * per);
  hi = min(n, lo + per);
}
// Exclusive block scan of one value per thread (256 threads); returns the
// block total through `total`.
__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v, unsigned long long& total) {
  __shared__ unsigned long long warp_sums[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  unsigned long long before = 0;
  total = 0;
  for (int w = 0; w < 8; ++w) {
    if (w < warp) before += warp_sums[w];
    total += warp_sums[w];
  }
  __syncthreads();  // warp_sums is reused by the next call
  return before + inc - v;
}
__global__ void __launch_bounds__(256) k_raster_scan_sums(RasterStream S) {
  uint32_t lo, hi;
  scan_range(S.count[1], lo, hi);
  unsigned long long sum = 0, total;
  for (uint32_t k = lo + threadIdx.x; k < hi; k += blockDim.x) sum += S.large_tiles[k];
  block_exclusive_scan(sum, total);
  if (threadIdx.x == 0) S.block_sums[blockIdx.x] = total;
}
__global__ void __launch_bounds__(256) k_raster_scan_top(RasterStream S) {
  unsigned long long total;
  const unsigned long long v = threadIdx.x < kRasterScanBlocks ? S.block_sums[threadIdx.x] : 0;
  const unsigned long long before = block_exclusive_scan(v, total);
  if (threadIdx.x < kRasterScanBlocks) S.block_sums[threadIdx.x] = before;
  if (threadIdx.x == 0) S.tile_prefix[S.count[1]] = total;
}
__global__ void __launch_bounds__(256) k_raster_scan_apply(RasterStream S) {
  uint32_t lo, hi;
  scan_range(S.count[1], lo, hi);
  unsigned long long carry = S.block_sums[blockIdx.x];
  for (uint32_t base = lo; base < hi; base += blockDim.x) {
    const uint32_t k = base + threadIdx.x;
    const unsigned long long v = k < hi ? S.large_tiles[k] : 0;
    unsigned long long total;
    const unsigned long long before = block_exclusive_scan(v, total);
    if (k < hi) S.tile_prefix[k] = carry + before;
    carry += total;
  }
}

// The large triangles' work items (blocks of 256 x 32 pixels of their
// bounding boxes), taken by warps from a ticket kRasterItemsPerTicket at a
// time (the first item's triangle by binary search of the prefix, the next
// ones by walking on); blocks the edge equations reject are skipped.
__global__ void __launch_bounds__(256) k_raster_depth_tiles(RasterStream S, ImageLayout L,
                                                            unsigned long long* __restrict__ depth_key) {
  const uint32_t n = S.count[1];
  if (n == 0) return;
  const unsigned long long total = S.tile_prefix[n];
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long w0 = 0;
    if (lane == 0)  // 64-bit ticket in count[2..3] (8-byte aligned): it cannot wrap below total
      w0 = atomicAdd(reinterpret_cast<unsigned long long*>(S.count + 2), (unsigned long long)kRasterItemsPerTicket);
    w0 = __shfl_sync(0xffffffffu, w0, 0);
    if (w0 >= total) break;
    const unsigned long long w1 = min(w0 + kRasterItemsPerTicket, total);
    uint32_t k = 0, hi = n - 1;  // last k with prefix[k] <= w0
    while (k < hi) {
      const uint32_t mid = (k + hi + 1) >> 1;
      if (S.tile_prefix[mid] <= w0) k = mid; else hi = mid - 1;
    }
    unsigned long long first = S.tile_prefix[k], next = S.tile_prefix[k + 1];
    for (unsigned long long w = w0; w < w1; ++w) {
      while (w >= next) {
        ++k;
        first = next;
        next = S.tile_prefix[k + 1];
      }
      const uint32_t q = S.large[k];
      const RasterSetup T = load_setup(S.tris + q);
      const Box b = bbox(T, L);
      const int rows = (b.y1 - b.y0 + kRasterTileH) / kRasterTileH;
      const int t = int(w - first);
      const int tx = t / rows, ty = t % rows;
      const int xs = b.x0 + tx * kRasterTileW, xe = min(xs + kRasterTileW - 1, b.x1);
      const int ys = b.y0 + ty * kRasterTileH, ye = min(ys + kRasterTileH - 1, b.y1);
      if (tile_outside(T, xs, xe, ys, ye)) continue;
      warp_block(T, q, xs, xe, ys, ye, L.height, depth_key);
    }
  }
}

__device__ __forceinline__ r3 mix3(r3 a, r3 b, float t) { return radd(rscale(a, sub(1.0f, t)), rscale(b, t)); }
__device__ __forceinline__ float clamp01(float x) { return fmn(fmx(x, 0.0f), 1.0f); }

// _height_band :976-1006
__device__ r3 height_band(float h) {
  const r3 deep = R3(0.015f, 0.12f, 0.34f), shallow = R3(0.02f, 0.63f, 0.82f), beach = R3(0.82f, 0.78f, 0.48f);
  const r3 lowland = R3(0.16f, 0.58f, 0.22f), upland = R3(0.48f, 0.42f, 0.16f), rock = R3(0.43f, 0.39f, 0.35f);
  const r3 snow = R3(0.94f, 0.96f, 0.98f);
  if (h < -250.0f) return mix3(deep, shallow, clamp01(dv(add(h, 5000.0f), 4750.0f)));
  if (h < 0.0f) return shallow;
  if (h < 120.0f) return mix3(beach, lowland, clamp01(dv(h, 120.0f)));
  if (h < 1400.0f) return mix3(lowland, upland, clamp01(dv(sub(h, 120.0f), 1280.0f)));
  if (h < 3000.0f) return mix3(upland, rock, clamp01(dv(sub(h, 1400.0f), 1600.0f)));
  return mix3(rock, snow, clamp01(dv(sub(h, 3000.0f), 1400.0f)));
}

// _surface_color :1008-1058
__device__ r3 surface_color(float h, const float (&m)[4], int slot, int mode, const int32_t* slot_level) {
  const r3 fertile = R3(0.10f, 0.34f, 0.075f), arid = R3(0.44f, 0.31f, 0.13f), rock = R3(0.34f, 0.32f, 0.30f);
  const r3 snow = R3(0.92f, 0.95f, 0.98f), sand = R3(0.72f, 0.60f, 0.34f);
  const r3 deep_ocean = R3(0.012f, 0.055f, 0.16f), shallow_ocean = R3(0.015f, 0.34f, 0.46f);
  r3 color = radd(radd(radd(rscale(fertile, m[0]), rscale(arid, m[1])), rscale(rock, m[2])), rscale(snow, m[3]));
  if (h < 0.0f) {
    color = mix3(shallow_ocean, deep_ocean, clamp01(dv(-h, 4200.0f)));
  } else if (h < 140.0f) {
    color = mix3(sand, color, clamp01(dv(h, 140.0f)));
  }
  if (mode == 1) {
    color = height_band(h);
  } else if (mode == 2) {
    const float hue = dv(float(slot_level[slot] % 6), 6.0f);
    const float h6 = mul(hue, 6.0f);
    color = R3(clamp01(sub(fabsf(sub(h6, 3.0f)), 1.0f)), clamp01(sub(2.0f, fabsf(sub(h6, 2.0f)))),
               clamp01(sub(2.0f, fabsf(sub(h6, 4.0f)))));
  } else if (mode == 3) {
    const float value = dv(float((int32_t(uint32_t(slot) * 1103515245u + 12345u)) & 255), 255.0f);
    const float a = add(mul(value, 0.73f), 0.21f), b = add(mul(value, 0.37f), 0.61f);
    color = R3(value, sub(a, floorf(a)), sub(b, floorf(b)));
  }
  return color;
}

// _resolve_raster :1208-1267
__global__ void __launch_bounds__(256) k_raster_resolve(RasterStream S, ImageLayout L,
                                                        const unsigned long long* __restrict__ depth_key,
                                                        RasterOutDev O, int mode, int triangles_per_patch,
                                                        const int32_t* __restrict__ slot_level) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)L.width * L.height) return;
  int x, y;
  if (L.sy <= L.sx) {  // y contiguous: the reference's (W, H, ...) layout
    x = int(i / L.height);
    y = int(i % L.height);
  } else {
    y = int(i / L.width);
    x = int(i % L.width);
  }
  const long long e = (long long)x * L.sx + (long long)y * L.sy;
  const unsigned long long key = depth_key[size_t(x) * L.height + y];
  if (key == kSentinel) {
    O.surface_id[e] = -1;
    O.cell_id[e] = -1;
    if (O.t_surface_id) O.t_surface_id[e] = -1;
    return;
  }
  const float z = __uint_as_float(uint32_t(key >> 32));
  TriBits u;
  const float4* rec = reinterpret_cast<const float4*>(S.tris + (key & 0xffffffffull));
#pragma unroll
  for (int k = 0; k < int(sizeof(RasterTri) / 16); ++k) u.v[k] = rec[k];
  const RasterTri& T = u.t;
  const r3 l = rscale(edge_values(T.s, add(float(x), 0.5f), add(float(y), 0.5f)), T.s.inv_area);
  const float w0 = dv(mul(l.x, z), T.s.screen[0][2]), w1 = dv(mul(l.y, z), T.s.screen[1][2]),
              w2 = dv(mul(l.z, z), T.s.screen[2][2]);
  auto lerp3 = [&](const float (&a)[3][3]) {
    return radd(radd(rscale(R3(a[0][0], a[0][1], a[0][2]), w0), rscale(R3(a[1][0], a[1][1], a[1][2]), w1)),
                rscale(R3(a[2][0], a[2][1], a[2][2]), w2));
  };
  const r3 bp = lerp3(T.v);
  const r3 bn = rnormalized(lerp3(T.n));
  float bm[4];
  for (int j = 0; j < 4; ++j) bm[j] = add(add(mul(T.m[0][j], w0), mul(T.m[1][j], w1)), mul(T.m[2][j], w2));
  const float bh = add(add(mul(T.h[0], w0), mul(T.h[1], w1)), mul(T.h[2], w2));
  int vi = 0;
  float wv = w0;
  if (w1 > w0) vi = 1, wv = w1;
  if (w2 > wv) vi = 2;
  const int32_t src = T.src;
  const r3 albedo = surface_color(bh, bm, src / triangles_per_patch, mode, slot_level);
  const int c = L.channels;
  O.depth[e] = z;
  O.surface_id[e] = src;
  O.cell_id[e] = vi == 0 ? T.c[0] : (vi == 1 ? T.c[1] : T.c[2]);  // constant indices keep the record in registers
  O.position[e * c + 0] = bp.x, O.position[e * c + 1] = bp.y, O.position[e * c + 2] = bp.z;
  O.normal[e * c + 0] = bn.x, O.normal[e * c + 1] = bn.y, O.normal[e * c + 2] = bn.z;
  O.albedo[e * c + 0] = albedo.x, O.albedo[e * c + 1] = albedo.y, O.albedo[e * c + 2] = albedo.z;
  for (int j = 0; j < 4; ++j) O.material[e * 4 + j] = bm[j];
  O.height[e] = bh;
  if (O.t_surface_id) {  // _snapshot_terrain_gbuffer, fused
    O.t_surface_id[e] = src;
    O.t_position[e * c + 0] = bp.x, O.t_position[e * c + 1] = bp.y, O.t_position[e * c + 2] = bp.z;
    O.t_normal[e * c + 0] = bn.x, O.t_normal[e * c + 1] = bn.y, O.t_normal[e * c + 2] = bn.z;
    O.t_albedo[e * c + 0] = albedo.x, O.t_albedo[e * c + 1] = albedo.y, O.t_albedo[e * c + 2] = albedo.z;
  }
}

__global__ void k_raster_clear(unsigned long long* __restrict__ depth_key, long long n, uint32_t* count) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < 4) count[i] = 0u;
  if (i < n) depth_key[i] = kSentinel;
}

}  // namespace

cudaError_t launch_raster(const RasterMeshDev& M, const RasterStream& S, const ImageLayout& L,
                          unsigned long long* depth_key, const RasterOutDev& O, float near, float tf, int mode,
                          int sm_count, cudaStream_t s) {
  const long long pixels = (long long)L.width * L.height;
  k_raster_clear<<<unsigned((pixels + 255) / 256), 256, 0, s>>>(depth_key, pixels, S.count);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long long sources = (long long)M.n_active * M.triangles_per_patch;
  if (sources > 0) {
    k_raster_clip<<<unsigned((sources + 127) / 128), 128, 0, s>>>(M, S, near, tf, L.width, L.height);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  k_raster_depth<<<unsigned(sm_count * 8), 256, 0, s>>>(S, L, depth_key);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_raster_scan_sums<<<kRasterScanBlocks, 256, 0, s>>>(S);
  k_raster_scan_top<<<1, 256, 0, s>>>(S);
  k_raster_scan_apply<<<kRasterScanBlocks, 256, 0, s>>>(S);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_raster_depth_tiles<<<unsigned(sm_count * 8), 256, 0, s>>>(S, L, depth_key);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_raster_resolve<<<unsigned((pixels + 255) / 256), 256, 0, s>>>(S, L, depth_key, O, mode, M.triangles_per_patch,
                                                                  M.slot_level);
  return cudaGetLastError();
}

}  // namespace atm
