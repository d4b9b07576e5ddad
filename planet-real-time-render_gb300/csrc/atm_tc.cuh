// atm_tc.cuh - 5th-generation tensor core (tcgen05) building blocks for the
// MLP networks on sm_103a: tensor-memory allocation, BF16 MMAs with the A
// operand in tensor memory and the B operand (weights) in shared memory,
// completion through an mbarrier, tensor-memory loads and stores for the
// per-row epilogue.  All inline PTX of the tcgen05 family lives here.
//
// Conventions of this file:
//  * one tile = 128 rows (samples / pixels) held by the 128 threads of four
//    consecutive warps; thread t of the tile owns TMEM lane t;
//  * a TMEM address is (lane << 16) | column; columns are 32 bit wide;
//  * the A operand of an MMA (M = 128 rows x K = 16 BF16) occupies 8
//    consecutive columns, each holding BF16 k = 2c (low half) and 2c + 1;
//  * weights of one layer: K-major, in 8 x 16-byte core matrices (8 output
//    neurons x 8 inputs); for MMA k-step s the core matrix of neuron group j
//    and input half i sits at ((s * NG + j) * 2 + i) * 128 bytes (NG = N / 8):
//    K-adjacent core matrices 128 B apart (LBO), N-adjacent 256 B (SBO).
#pragma once

#include <cstdint>

namespace atm {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- tensor memory ----------------------------------------------------------
// Whole-warp operations.  The allocated base address is written to *dst.
__device__ __forceinline__ void alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- descriptors ---------------------------------------------------------------
// Shared-memory matrix descriptor, no swizzle (bits 0-13 start >> 4, 16-29
// leading byte offset >> 4, 32-45 stride byte offset >> 4, 46-47 version 1,
// 61-63 layout 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFFu);
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;
  return d;
}
// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

// ---- MMA -------------------------------------------------------------------------
// D[tmem] (+)= A[tmem] x B[smem]; one thread issues.
__device__ __forceinline__ void mma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive on the mbarrier when every MMA this thread issued so far is done.
__device__ __forceinline__ void commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
               : "memory");
}

// ---- mbarrier ------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Waits for the phase with the given parity; gives up after max_tries polls
// (each try_wait itself suspends for a bounded time) and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, int max_tries) {
  const uint32_t a = smem_addr(mbar);
  for (int i = 0; i < max_tries; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Arrival of the calling thread that also expects `bytes` of transactions.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(bytes)
               : "memory");
}

// ---- bulk copy (the TMA engine's untiled form) -----------------------------------
// global -> this CTA's shared memory; completes `bytes` of transactions on
// mbar.  Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(static_cast<uint64_t>(__cvta_generic_to_global(src))), "r"(bytes), "r"(smem_addr(mbar))
      : "memory");
}

// ---- tensor-memory loads and stores (32 lanes x 32 bit per warp) ----------------
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void st8(uint32_t taddr, const uint32_t (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(v[0]),
               "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
               : "memory");
}
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Named barrier over the 128 threads of one tile (ids 1..).
__device__ __forceinline__ void tile_sync(int tile) {
  asm volatile("bar.sync %0, 128;" ::"r"(tile + 1) : "memory");
}
// The same barrier, returning whether v holds in every thread of the tile:
// a bounded wait can end true in one thread and false in another, and the
// tile must take one path afterwards (its barriers stay matched).
__device__ __forceinline__ bool tile_all(int tile, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, %2, 128, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"(uint32_t(v)), "r"(tile + 1)
      : "memory");
  return r != 0;
}

}  // namespace tc
}  // namespace atm
