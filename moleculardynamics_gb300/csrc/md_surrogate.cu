// Learned surrogate of the bond-order term (common/arvdwfc + the bond-order
// functions of cpu/common/BondOrderFuncs.h): per-atom Behler symmetry
// functions (16 radial, 16 angular, FP32), a 32-64-64-1 MLP with BF16
// weights on the tensor cores (tcgen05, FP32 accumulation in tensor memory),
// forces from the network's analytic gradient, Adam training on per-atom
// energies of the exact method.  This file starts with the tensor-core GEMM
// building block and its self-test.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/mdgb.h"
#include "md_internal.h"
#include "md_tc.cuh"

namespace mdgb {

namespace {

constexpr int kTcThreads = 128;

// C[128 x N] = A[128 x K] * B[N x K]^T on the tensor cores (one CTA); A, B
// row-major FP32 in global memory, rounded to BF16 on the way into shared
// memory.  Dynamic shared memory: A at 0, B at 64 KB.
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_selftest(const float* __restrict__ A, const float* __restrict__ B,
                  float* __restrict__ C, int N, int K, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* As = sm;
  unsigned char* Bs = sm + 65536;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_taddr;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int e = tid; e < 128 * K; e += blockDim.x) {
    const int r = e / K, k = e % K;
    *(__nv_bfloat16*)(As + tc_offset(r, k, K)) = __float2bfloat16_rn(A[e]);
  }
  for (int e = tid; e < N * K; e += blockDim.x) {
    const int r = e / K, k = e % K;
    *(__nv_bfloat16*)(Bs + tc_offset(r, k, K)) = __float2bfloat16_rn(B[e]);
  }
  fence_proxy_async();  // generic-proxy writes before the tensor core reads them
  const uint32_t ncols = N <= 32 ? 32u : (N <= 64 ? 64u : 128u);
  if (warp == 0) tc_alloc(&s_taddr, ncols);
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t taddr = s_taddr;
  if (tid == 0) tc_gemm_issue(taddr, As, Bs, N, K, &bar);
  const bool ok = mbar_wait(&bar, 0u, status);
  tc_fence_after();
  if (__syncthreads_and(ok)) {
    const int row = 32 * warp + (tid & 31);
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc_ld16(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int k = 0; k < 16; k++) C[row * N + c0 + k] = v[k];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(taddr, ncols);
}

}  // namespace

}  // namespace mdgb

using namespace mdgb;

extern "C" {

// Tensor-core self-test: C[128 x N] = A[128 x K] * B[N x K]^T with BF16
// operands (rounded to nearest even from the FP32 inputs) and FP32
// accumulation.  N in {32, 64, 128}, K a multiple of 16 up to 128.
md_status mdgb_tc_selftest(const float* A, const float* B, float* C, int N, int K) {
  if (!A || !B || !C || !(N == 32 || N == 64 || N == 128) || K < 16 || K > 128 || K % 16)
    return MD_BAD_ARGUMENT;
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int* dst = nullptr;
  cudaError_t e = cudaSuccess;
  auto done = [&](md_status s) {
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(dst);
    return s;
  };
  if ((e = cudaMalloc(&dA, sizeof(float) * 128 * K)) != cudaSuccess ||
      (e = cudaMalloc(&dB, sizeof(float) * N * K)) != cudaSuccess ||
      (e = cudaMalloc(&dC, sizeof(float) * 128 * N)) != cudaSuccess ||
      (e = cudaMalloc(&dst, sizeof(int))) != cudaSuccess)
    return done(MD_OUT_OF_MEMORY);
  cudaMemcpy(dA, A, sizeof(float) * 128 * K, cudaMemcpyHostToDevice);
  cudaMemcpy(dB, B, sizeof(float) * N * K, cudaMemcpyHostToDevice);
  cudaMemset(dst, 0, sizeof(int));
  const int smem = 65536 + 65536;
  cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_tc_selftest<<<1, kTcThreads, smem>>>(dA, dB, dC, N, K, dst);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return done(MD_CUDA_ERROR);
  int st = 0;
  cudaMemcpy(&st, dst, sizeof(int), cudaMemcpyDeviceToHost);
  cudaMemcpy(C, dC, sizeof(float) * 128 * N, cudaMemcpyDeviceToHost);
  return done(st ? MD_TIMEOUT : MD_OK);
}

}  // extern "C"
