// TMA (cp.async.bulk.tensor) and mbarrier helpers in inline PTX for sm_103a.
//
// A tile copy is issued by one thread: mbarrier.arrive.expect_tx announces
// the bytes, cp.async.bulk.tensor.2d moves the tile into shared memory and
// completes the transaction on the mbarrier.  Consumers wait on the barrier
// phase with a bounded loop; a wait that runs out records ST_TMA_TIMEOUT in
// the status word and the kernel returns instead of spinning forever.
#pragma once
#include <cuda.h>
#include <stdint.h>

#include "md_internal.h"

namespace mdgb {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// 2-D tiled tensor load: box at coordinates (x, y) into dst, completing on bar
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// 1-D bulk copy global -> shared (both 16-byte aligned, bytes a multiple of
// 16), completing on bar
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"((unsigned long long)src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of bar: at most `limit` polls (a kernel
// argument; 0 gives up at once).  Returns false (and flags the status word)
// when the limit runs out.
constexpr int kWaitLimit = 1 << 20;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status,
                                          int limit = kWaitLimit) {
  for (int it = 0; it < limit; it++)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(status, ST_TMA_TIMEOUT);
  return false;
}

// try_wait with a suspend-time hint: the warp may sleep up to hint_ns in the
// instruction instead of returning at once, so a long wait issues few polls
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity,
                                                    uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// mbar_wait with sleeping polls (waits of whole blocks on staged copies);
// at most `limit` polls of up to kWaitHintNs each
constexpr uint32_t kWaitHintNs = 2000;
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, int* status,
                                                int limit = kWaitLimit) {
  for (int it = 0; it < limit; it++)
    if (mbar_try_wait_sleep(bar, parity, kWaitHintNs)) return true;
  atomicOr(status, ST_TMA_TIMEOUT);
  return false;
}

// After a wait gave up: the copies this block still has in flight land in
// its shared memory before it leaves.  Always the default limit, whatever
// limit the failed wait had, so that no copy outlives the block.
__device__ __forceinline__ bool mbar_drain(uint64_t* bar, uint32_t parity, int* status) {
  return mbar_wait(bar, parity, status, kWaitLimit);
}

// L2 prefetch of one box of a tiled tensor map (coordinates as for
// tma_load_2d; no shared memory, no barrier, no completion to wait for)
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap* map, int x, int y) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(
                   (unsigned long long)map),
               "r"(x), "r"(y)
               : "memory");
}

// L2 prefetch of the line holding p (no register result, no wait)
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

}  // namespace mdgb
