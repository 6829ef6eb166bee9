// Fifth-generation tensor cores (tcgen05) for the CTA-level contractions.
//
// One elected thread issues tcgen05.mma; A and B are read from shared memory
// through matrix descriptors, the FP32 accumulator D lives in tensor memory
// (TMEM) and is read back by the CTA with tcgen05.ld.  Completion of the MMAs
// is signalled on an mbarrier by tcgen05.commit.
//
// Operand tiles use the canonical K-major layout without swizzling: the tile
// is cut into core matrices of 8 rows x 16 bytes (8 x 8 BF16 or 8 x 4 TF32),
// each stored as 128 contiguous bytes (row r of the core matrix at byte 16 r).
// Core matrices adjacent along K are LBO = 128 bytes apart; groups of 8 rows
// are SBO = (K bytes / 16) * 128 bytes apart.  One MMA consumes 32 bytes of K
// (K = 16 BF16 or K = 8 TF32): its descriptor starts 256 bytes further for
// every K step.
//
// Accumulator layout (M = 128, cta_group::1): row i of D is TMEM lane i,
// column j of D is TMEM column (base + j), one 32-bit value each.  Warp w of
// the CTA may read lanes 32 (w % 4) .. 32 (w % 4) + 31 only.
//
// Every wait is bounded (ttals_device.cuh); a wait that gives up reports
// ST_TIMEOUT and the caller leaves without touching the accumulator.
#pragma once

#include <stdint.h>

#include "ttals_device.cuh"

namespace ttals {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- instruction descriptors (kind::f16 with BF16 inputs, kind::tf32) -------

// bits: [4,6) D format (1 = F32), [7,10) A format, [10,13) B format
// (kind::f16: 1 = BF16; kind::tf32: 2 = TF32), [15] A MN-major, [16] B MN-major
// (both 0: K-major), [17,23) N >> 3, [24,29) M >> 4.
__host__ __device__ constexpr uint32_t idesc(uint32_t ab_format, int M, int N) {
  return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
constexpr uint32_t kFmtBF16 = 1;
constexpr uint32_t kFmtTF32 = 2;

// ---- shared-memory matrix descriptor (no swizzle, K-major) -------------------

// bits: [0,14) start address >> 4, [16,30) leading-dimension byte offset >> 4,
// [32,46) stride-dimension byte offset >> 4, [46,48) version = 1, [49,52) base
// offset = 0, [52] LBO mode = 0, [61,64) layout = 0 (no swizzle).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// Byte offset of element (r, k) in a K-major no-swizzle tile whose rows hold
// kbytes bytes of K (a multiple of 32); esz = element size (2 or 4).
__host__ __device__ __forceinline__ uint32_t tile_off(int r, int k, int esz, int kbytes) {
  const int per = 16 / esz;  // elements per 16-byte core-matrix row
  const int chunk = k / per, within = k - chunk * per;
  return (uint32_t)((r >> 3) * (kbytes / 16) * 128 + chunk * 128 + (r & 7) * 16 + within * esz);
}

// ---- TMEM allocation (one warp) ----------------------------------------------

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- fences --------------------------------------------------------------------

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes (st.shared) -> visible to the tensor cores
__device__ __forceinline__ void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- MMA ------------------------------------------------------------------------

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate)
      : "memory");
}

// Arrive (once) on the mbarrier when every MMA this thread issued so far is done.
__device__ __forceinline__ void commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

// ---- mbarrier -------------------------------------------------------------------

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of the mbarrier; false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit = 1u << 24) {
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(mbar, parity)) return true;
  return false;
}

// ---- TMEM -> registers ------------------------------------------------------------

// 16 consecutive 32-bit columns of this thread's lane (warp-collective).
__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// TMEM address of (lane, column) relative to the allocation base.
__device__ __forceinline__ uint32_t taddr(uint32_t base, int lane, int col) {
  return base + ((uint32_t)lane << 16) + (uint32_t)col;
}

}  // namespace umma
}  // namespace ttals
