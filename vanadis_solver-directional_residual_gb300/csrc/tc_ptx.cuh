// tc_ptx.cuh -- thin inline-PTX wrappers for the Blackwell (sm_100 family)
// asynchronous data path: mbarriers, TMA tensor and bulk copies, and the
// fifth-generation tensor cores (tcgen05: MMA from shared-memory
// descriptors into tensor memory, TMEM allocation and loads).
//
// Every wait is bounded: mbar_wait gives up after `limit` clock cycles and
// reports it, so that a kernel whose data never arrives sets an error flag
// and returns instead of spinning.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace vdr {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// ------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
// Makes the initialised barriers visible to the async proxy (TMA, tcgen05).
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n"
      " selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// try_wait with a suspend-time hint: the thread sleeps until the phase
// completes or about `hint_ns` nanoseconds pass, instead of returning at
// once, so that waiting warps leave the issue slots to the working ones.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint32_t bar, uint32_t parity,
                                                    uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}
// Waits as mbar_wait below, sleeping in the try_wait between checks of the
// clock (each sleep at most `hint_ns`, far below the limit).
__device__ __forceinline__ bool mbar_wait_sleep(uint32_t bar, uint32_t parity, long long limit,
                                                uint32_t hint_ns = 20000u) {
  if (mbar_try_wait_sleep(bar, parity, hint_ns)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait_sleep(bar, parity, hint_ns))
    if (clock64() - t0 > limit) return false;
  return true;
}
// Waits until the phase with the given parity has completed, at most
// `limit` cycles; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
                                          long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}

// ------------------------------------------------------------- TMA
// 4-D tiled tensor load into shared memory, completion on `bar`.
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map,
                                            int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}
// Plain bulk copy global -> shared (16-byte aligned, size a multiple of 16).
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"((uint64_t)src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

// ------------------------------------------------------------- tcgen05
// Shared-memory matrix descriptor, no swizzle (the canonical "interleaved"
// K-major layout: core matrices of 8 rows x 16 bytes, rows 16 bytes apart):
// lbo = byte distance between core matrices adjacent in K, sbo = between
// core matrices adjacent in M (or N).  Fields: start address >> 4 in bits
// 0-13, lbo >> 4 in 16-29, sbo >> 4 in 32-45, the fixed value 1 in bits
// 46-47, base offset 0, swizzle mode 0 (none) in bits 61-63.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
// Swizzled K-major descriptor (layout 2 = 128B, 4 = 64B, 6 = 32B swizzle):
// rows of the swizzle width, consecutive 8-row groups `sbo` bytes apart;
// the leading offset is unused (an MMA's K extent lies within one row).
// The swizzle is applied to absolute shared-memory address bits, as the TMA
// unit applies it, so the start may lie anywhere on a 16-byte boundary
// inside a slab the TMA unit wrote with the same mode (base offset 0).
__device__ __forceinline__ uint64_t smem_desc_sw(uint32_t addr, uint32_t sbo, int layout) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)(layout & 7) << 61;
  return d;
}
// Instruction descriptor of kind::f16 with BF16 A and B, FP32 accumulator,
// both operands K-major: D format (1 = F32) in bits 4-5, A format (1 =
// BF16) in 7-9, B format in 10-12, N >> 3 in 17-22, M >> 4 in 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
// D[tmem] (+)= A[adesc] * B[bdesc]^T, one CTA, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The barrier receives one arrive once every tcgen05 operation this thread
// issued before has completed.
__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
// Whole warp: allocates `cols` TMEM columns (a power of two >= 32) and writes
// the address to shared memory at `slot`.
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
               "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols)
               : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
// Whole warp: 16 consecutive 32-bit columns of the warp's 32 TMEM lanes
// (thread i <- lane base + i).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

}  // namespace tc
}  // namespace vdr
