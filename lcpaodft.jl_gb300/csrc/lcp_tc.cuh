// tcgen05 building blocks for sm_103a: tensor-memory allocation, shared-memory
// matrix descriptors (no-swizzle canonical layouts), the kind::f16 instruction
// descriptor, MMA issue/commit, bounded mbarrier waits and TMEM loads.
//
// Canonical no-swizzle layouts (16-bit elements, "core matrix" = 8 x 8
// elements = 128 contiguous bytes):
//   K-major  operand (rows = M or N, K contiguous in 16-byte row pieces):
//       byte(r, k)  = (r/8)*SBO + (k/8)*LBO + ((r%8)*8 + k%8)*2
//   MN-major operand (M or N contiguous in 16-byte pieces along K rows):
//       byte(mn, k) = (mn/8)*SBO + (k/8)*LBO + ((k%8)*8 + mn%8)*2
// SBO strides the 8-groups along M/N, LBO the 8-groups along K.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace lcp {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, LBO, SBO (bytes, multiples
// of 16), descriptor version 1, base offset 0, SWIZZLE_NONE.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// Instruction descriptor of tcgen05.mma .kind::f16 with BF16 A/B and an FP32
// accumulator; a_mn / b_mn select the MN-major ("transposed") operand layout.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N, int a_mn, int b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(a_mn) << 15) |
         (static_cast<uint32_t>(b_mn) << 16) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

// ---------------------------------------------------------------- TMEM

// Executed by one full warp.  Writes the TMEM base address to *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes generic-proxy shared-memory writes visible to the tensor core.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------- MMA

// One lane of the converged warp, chosen by elect.sync; for the same member
// mask it is the same lane every time.
__device__ __forceinline__ bool elect_one() {
  uint32_t pred = 0;
  asm volatile(
      "{\n\t.reg .pred P;\n\t"
      "elect.sync _|P, 0xffffffff;\n\t"
      "selp.u32 %0, 1, 0, P;\n\t}"
      : "=r"(pred));
  return pred != 0;
}

// D[tmem] (+)= A[smem] * B[smem]; issued by a single thread.
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives (once) on the mbarrier when all MMAs issued so far by this thread finish.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

// ---------------------------------------------------------------- mbarrier

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
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

// Non-blocking probe of the phase.  Every wait below probes with it first:
// per-step clock64 traces showed ~200 cycles spent in waits whose phase had
// completed long before, and the probe took the density kernel's stage from
// 0.511 to 0.489 ms on the 64-atom cell (the grid-H stage did not change).
__device__ __forceinline__ bool mbar_test_wait(uint64_t* mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: returns false when the phase did not complete within
// max_iters polls (the caller records an error and unwinds).
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_iters = (1u << 26)) {
  if (mbar_test_wait(mbar, parity)) return true;
  for (uint32_t i = 0; i < max_iters; ++i)
    if (mbar_try_wait(mbar, parity)) return true;
  return false;
}

// Bounded wait that also gives up as soon as *abort is set by another role of
// the CTA.  Returns false on timeout or abort.
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t* mbar, uint32_t parity, const volatile int* abort,
                                                    uint32_t max_iters = (1u << 24)) {
  if (mbar_test_wait(mbar, parity)) return true;
  for (uint32_t i = 0; i < max_iters; ++i) {
    if (mbar_try_wait(mbar, parity)) return true;
    if ((i & 63u) == 63u && *abort) return false;
  }
  return false;
}

// The abortable wait with one outcome for the whole warp (for warps that
// then issue through elect.sync, which needs the converged warp).
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* mbar, uint32_t parity, const volatile int* abort,
                                               uint32_t max_iters = (1u << 24)) {
  return __all_sync(0xffffffffu, mbar_wait_abortable(mbar, parity, abort, max_iters)) != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// Arrives once and adds `bytes` to the phase's expected transaction count.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
               : "memory");
}

// ---------------------------------------------------------------- bulk copies (TMA, untiled)

// global -> shared copy of `bytes` (multiple of 16; both addresses 16-byte
// aligned), completing as transactions on the mbarrier.
__device__ __forceinline__ void bulk_g2s(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(sdst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}

// Barrier among `nthreads` threads (whole warps) of the CTA.
__device__ __forceinline__ void named_bar_sync(uint32_t id, uint32_t nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// ---------------------------------------------------------------- TMEM -> registers

// 32 lanes x 16 consecutive 32-bit columns: thread t of the warp receives lane
// (warp's lane quarter + t), columns [col, col+16).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// The same load without waiting: several loads can be in flight before one
// tmem_wait_ld(); the registers are valid only after it.
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// Ties 16 loaded registers to a point after tmem_wait_ld(): the compiler sees
// them redefined here, so no use of them is scheduled before the wait.
__device__ __forceinline__ void tmem_regs_ready(uint32_t* r) {
  asm volatile(""
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]));
}

// TMEM address of (lane, column): lane in bits 31..16, column in bits 15..0.
__device__ __forceinline__ uint32_t tmem_addr(uint32_t base, uint32_t lane, uint32_t col) {
  return base + (lane << 16) + col;
}

// ---------------------------------------------------------------- canonical offsets

__device__ __forceinline__ uint32_t kmajor_off(uint32_t r, uint32_t k, uint32_t lbo, uint32_t sbo) {
  return (r >> 3) * sbo + (k >> 3) * lbo + (((r & 7) << 3) + (k & 7)) * 2;
}
__device__ __forceinline__ uint32_t mnmajor_off(uint32_t mn, uint32_t k, uint32_t lbo, uint32_t sbo) {
  return (mn >> 3) * sbo + (k >> 3) * lbo + (((k & 7) << 3) + (mn & 7)) * 2;
}


}  // namespace tc
}  // namespace lcp
