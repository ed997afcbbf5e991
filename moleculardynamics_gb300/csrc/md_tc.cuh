// 5th-generation tensor-core (tcgen05) helpers in inline PTX for sm_103a.
//
// A CTA of 128 threads computes D[128 x N] (FP32, in tensor memory) =
// A[128 x K] * B[N x K]^T from BF16 operands in shared memory:
//   - operands are stored K-major without swizzle as 8-row x 16-byte "core
//     matrices" (8 x 8 BF16): element (r, k) of an R x K tile sits at byte
//     (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2, with
//     LBO = 128 (core matrices adjacent along K) and SBO = K * 16;
//   - one warp allocates tensor-memory columns (tcgen05.alloc), one thread
//     issues tcgen05.mma (M = 128, K = 16 per instruction, FP32 accumulate)
//     and tcgen05.commit to an mbarrier;
//   - after the mbarrier completes, warp w reads rows 32w .. 32w+31 with
//     tcgen05.ld (shape 32x32b: one row per thread, consecutive columns).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "md_tma.cuh"

namespace mdgb {

// byte offset of element (r, k) in a K-major, unswizzled R x K BF16 tile
__host__ __device__ __forceinline__ uint32_t tc_offset(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start, LBO, SBO (bytes), no swizzle;
// bits 46-48 hold the fixed value 0b001 of the tcgen05 descriptor format
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M x N
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_alloc(uint32_t* smem_dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_addr(smem_dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D (tensor memory) (+)= A * B^T, one instruction (K = 16)
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                       uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// the mbarrier completes when every earlier tcgen05.mma of this thread is done
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_addr(bar))
      : "memory");
}

// 16 consecutive FP32 columns of this thread's row
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

// D[128 x N] (+)= A[128 x K] * B[N x K]^T with A and B in shared memory
// (layout above); issued by the calling thread; with bar, completion of all
// earlier products of this thread is signalled there
__device__ __forceinline__ void tc_gemm_issue(uint32_t d_tmem, const void* A, const void* B,
                                              int N, int K, uint64_t* bar,
                                              bool accumulate = false) {
  const uint32_t a0 = smem_addr(A), b0 = smem_addr(B);
  const uint32_t sbo = (uint32_t)K * 16u;
  const uint32_t idesc = tc_idesc_bf16(128, N);
  for (int j = 0; j < K / 16; j++) {
    // K = 16 per instruction: two core matrices along K
    tc_mma(d_tmem, tc_desc(a0 + j * 256u, 128u, sbo), tc_desc(b0 + j * 256u, 128u, sbo), idesc,
           accumulate || j > 0);
  }
  if (bar) tc_commit(bar);
}

}  // namespace mdgb
