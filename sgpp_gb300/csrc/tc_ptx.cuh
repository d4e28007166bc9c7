// Inline-PTX wrappers for the 5th-generation tensor cores of sm_100-family GPUs (tcgen05: MMA
// issued by one thread, accumulators in tensor memory), mbarriers with bounded waits, and the
// shared-memory matrix descriptors they read (internal to libsgpp_gb300).
//
// Operand layout (no swizzle): a matrix in shared memory is a grid of "core matrices" of 8 rows x
// 16 bytes (8 rows of eight 16-bit elements along the contiguous dimension), each stored as 128
// contiguous bytes; the descriptor gives the byte distances between neighbouring core matrices
// along the two dimensions. Accumulators of an M = 128 MMA occupy tensor-memory lanes 0..127 (one
// row each) and one 32-bit column per output column.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sgmev {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor, no swizzle: start address, then the byte offsets between core
// matrices along the leading (LBO) and the strided (SBO) dimension, descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) |
         (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (static_cast<uint64_t>(1) << 46);
}

// Instruction descriptor of tcgen05.mma kind::f16 with BF16 A and B, FP32 accumulation, dense;
// a_mn / b_mn select the MN-major (transposed) operand layouts.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n, bool a_mn, bool b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) |
         ((b_mn ? 1u : 0u) << 16) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}
// The same with FP16 A and B (type field 0 for both; A and B always share one type)
__host__ __device__ constexpr uint32_t idesc_f16(int m, int n, bool a_mn, bool b_mn) {
  return (1u << 4) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
         (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}

// ---- tensor memory ------------------------------------------------------------------------
// allocation and release are warp-wide (one warp, the same one for both)
__device__ __forceinline__ void tmem_alloc(uint32_t holder_saddr, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(holder_saddr),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes to shared memory become visible to the tensor cores' reads
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 lanes x 16 columns of 32 bits: thread i of the warp gets lane (warp % 4) * 32 + i
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 32 lanes x 32 columns of 32 bits from registers: thread i of the warp writes lane
// (warp % 4) * 32 + i
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]),
      "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]),
      "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]),
      "r"(r[30]), "r"(r[31])
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// D[tmem] (+)= A[tmem] B[smem], issued by one thread. A of an M = 128 MMA with 16-bit elements:
// lane m holds row m, column c the K elements 2c (low half) and 2c + 1 (high half).
__device__ __forceinline__ void mma_bf16_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc,
                                            uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u));
}

// D[tmem] (+)= A[smem] B[smem], issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u));
}
// the mbarrier completes one arrival when every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint32_t mbar_saddr) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          mbar_saddr)
      : "memory");
}

// True in one lane of the (converged) warp, the same lane every time while all 32 are active.
// The MMA warp runs its loop with all lanes and issues each MMA from the elected lane: MMAs issued
// by a lone thread of a diverged warp cost 2.5 times as much (measured at M = 128, N = 32), and a
// branch between two MMAs another factor of two.
__device__ __forceinline__ bool elect_one() {
  uint32_t pred = 0;
  asm volatile(
      "{\n.reg .pred P;\n.reg .b32 R;\nelect.sync R|P, 0xffffffff;\nselp.b32 %0, 1, 0, P;\n}\n"
      : "=r"(pred));
  return pred != 0;
}

// ---- mbarriers ----------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint32_t saddr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr), "r"(count));
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t saddr) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(saddr)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t saddr, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(saddr), "r"(parity)
      : "memory");
  return done != 0;
}
// non-blocking test of the same (never suspends the thread)
__device__ __forceinline__ bool mbar_poll(uint32_t saddr, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(saddr), "r"(parity)
      : "memory");
  return done != 0;
}
// Wait for the phase of the given parity to complete, at most `limit` polls (each try_wait
// suspends the thread for a while). Returns false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t saddr, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_test(saddr, parity)) return true;
  return false;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// try_wait that may suspend the thread for up to `hint_ns` while the phase is incomplete, so that
// waiting threads do not take issue slots from working ones
__device__ __forceinline__ bool mbar_test_suspend(uint32_t saddr, uint32_t parity, uint32_t hint_ns) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(saddr), "r"(parity), "r"(hint_ns)
      : "memory");
  return done != 0;
}
// Wait for the phase of the given parity to complete, for at most `limit_ns` nanoseconds of the
// global timer. Returns false when the time ran out.
__device__ __forceinline__ bool mbar_wait_ns(uint32_t saddr, uint32_t parity, uint64_t limit_ns) {
  if (mbar_test(saddr, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (;;) {
    if (mbar_test_suspend(saddr, parity, 20000u)) return true;
    if (globaltimer_ns() - t0 > limit_ns) return false;
  }
}

}  // namespace tc
}  // namespace sgmev
