/*
 * tl_tc05.cuh -- the fifth-generation tensor core (tcgen05) of sm_100/sm_103
 * from inline PTX: tensor-memory allocation, shared-memory matrix and
 * instruction descriptors, the single-thread MMA, its completion through an
 * mbarrier, and the tensor-memory loads of the epilogue.
 *
 * Shared-memory operands use the canonical K-major layout without swizzling:
 * a "core matrix" is 8 rows x 16 bytes (8 FP16 values of K), stored as 128
 * contiguous bytes; the descriptor's leading byte offset (LBO) is the
 * distance between the two core matrices that cover K = 0..7 and 8..15 of
 * one MMA, its stride byte offset (SBO) the distance between consecutive
 * 8-row groups along M (or N). With SBO = 128 the rows of one K chunk are
 * simply consecutive 16-byte slots, so moving the start address by 16 bytes
 * moves the operand down by one row.
 *
 * Every wait is bounded (%globaltimer): a wait that runs out reports
 * failure instead of spinning on.
 */
#pragma once

#include <stdint.h>

namespace tc05 {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

/* Shared-memory matrix descriptor: K-major, no swizzle, descriptor version 1
 * (bits 46-47), base offset 0, layout type 0. Addresses and offsets in bytes,
 * multiples of 16. */
__device__ __forceinline__ uint64_t smem_desc(uint32_t start, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((start >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

/* Instruction descriptor of kind::f16 with FP16 A and B, FP32 accumulator,
 * both operands K-major: D format at bits 4-5 (1 = F32), A/B formats at
 * 7-9 / 10-12 (0 = F16), N >> 3 at bits 17-22, M >> 4 at bits 24-28. */
template <int M, int N>
__host__ __device__ constexpr uint32_t idesc_f16_f32() {
  static_assert(M == 64 || M == 128, "M must be 64 or 128");
  static_assert(N % 8 == 0 && N >= 8 && N <= 256, "N must be a multiple of 8 in [8, 256]");
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/* Tensor-memory allocation of ncols columns (a power of two >= 32) by one
 * whole warp; the base address is written to *dst (shared memory). */
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
               :: "r"(smem_addr(dst)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
               :: "r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
/* Makes this thread's generic-proxy shared-memory writes visible to the
 * tensor core (async proxy). */
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

/* D (tensor memory) = A * B^T (+ D if accumulate), issued by one thread. */
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                        uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n"
      :: "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

/* The mbarrier receives one arrival when every MMA issued so far by this
 * thread has completed. */
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
      :: "r"(smem_addr(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n"
               :: "r"(smem_addr(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

/* Waits until the mbarrier phase with the given parity has completed, for at
 * most budget_ns; returns false if the wait ran out. */
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity,
                                          unsigned long long budget_ns) {
  const uint32_t addr = smem_addr(mbar);
  const unsigned long long t0 = now_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done) : "r"(addr), "r"(parity) : "memory");
    if (done) return true;
    if (now_ns() - t0 > budget_ns) return false;
  }
}

/* Two loads of 32 lanes x 16 columns of 32-bit values: thread t of the warp
 * receives lane (lane field of the address) + t, columns col .. col + 15 of
 * each address. The warp may only address the 32 lanes of its own
 * sub-partition (warp id % 4). tcgen05.ld is asynchronous: its destination
 * registers hold the values only after tcgen05.wait::ld, so the loads and the
 * wait are one asm statement; as two statements the compiler would see no
 * dependence of the destinations on the wait and could use them before it. */
__device__ __forceinline__ void tmem_ld16x2(uint32_t taddr_a, uint32_t taddr_b, float va[16],
                                            float vb[16]) {
  uint32_t a[16], b[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%32];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%33];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3]), "=r"(a[4]), "=r"(a[5]), "=r"(a[6]),
        "=r"(a[7]), "=r"(a[8]), "=r"(a[9]), "=r"(a[10]), "=r"(a[11]), "=r"(a[12]),
        "=r"(a[13]), "=r"(a[14]), "=r"(a[15]), "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3]),
        "=r"(b[4]), "=r"(b[5]), "=r"(b[6]), "=r"(b[7]), "=r"(b[8]), "=r"(b[9]), "=r"(b[10]),
        "=r"(b[11]), "=r"(b[12]), "=r"(b[13]), "=r"(b[14]), "=r"(b[15])
      : "r"(taddr_a), "r"(taddr_b)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    va[i] = __uint_as_float(a[i]);
    vb[i] = __uint_as_float(b[i]);
  }
}

}  // namespace tc05
