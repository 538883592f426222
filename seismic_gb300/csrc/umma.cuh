// umma.cuh - 5th-generation tensor-core (tcgen05) helpers for sm_103a.
//
// One elected thread issues tcgen05.mma with both operands in shared memory
// (BF16, K-major, no swizzle) and the FP32 accumulator in tensor memory
// (TMEM); completion is signalled on an mbarrier through tcgen05.commit and
// the epilogue reads the accumulator back with tcgen05.ld.
//
// Shared-memory operand layout (no swizzle, K-major): "core matrices" of
// 8 rows x 16 bytes (8 BF16 along K), rows 16 bytes apart.  For a tile of R
// rows the core matrix (r/8, k/8) starts at ((k/8) * (R/8) + r/8) * 128
// bytes, so core matrices adjacent along R are 128 bytes apart (the stride
// byte offset) and those adjacent along K are R/8 * 128 bytes apart (the
// leading byte offset).
#pragma once

#include <cstdint>

namespace swave {

__device__ __forceinline__ unsigned umma_su32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// Byte offset of element (r, k) of an R-row K-major BF16 tile.
__device__ __forceinline__ int umma_off(int r, int k, int R) {
  return (((k >> 3) * (R >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_alloc(unsigned *dst_smem, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   umma_su32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void umma_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void umma_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void umma_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes become visible to the tensor cores.
__device__ __forceinline__ void umma_fence_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T for one K = 16 slice.
__device__ __forceinline__ void umma_bf16(unsigned d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}
__device__ __forceinline__ void umma_commit(unsigned long long *mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          umma_su32(mbar))
      : "memory");
}
__device__ __forceinline__ void umma_mbar_init(unsigned long long *mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(umma_su32(mbar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Bounded wait on an mbarrier phase; false if it gave up.
__device__ __forceinline__ bool umma_mbar_wait(unsigned long long *mbar, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(umma_su32(mbar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void umma_ld16(unsigned taddr, float *out) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) out[q] = __uint_as_float(r[q]);
}

}  // namespace swave
