// Arithmetic peaks of the current GPU, measured with CUDA events.
//
// The HBM and tensor-core peaks of the roofline come from outside the
// library; the FP64 and FP32 pipe rates that bound the plain FP64 path, the
// Gear update and the bond-order kernels are measured here with dependent
// FMA chains: every thread runs kChains independent chains (enough to cover
// the pipe latency), and the grid fills every SM several times.  The result
// is FMA operations per second x 2 (flops).
#include <cuda_runtime.h>

#include "../../include/mdgb.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kThreads) k_fma_chains(T* out, int iters, T a, T b) {
  T x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = (T)(threadIdx.x + k) * (T)1e-6;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = fma(x[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += x[k];
  // never true for the arguments used (the chains converge to b / (1 - a) > 0);
  // keeps the chains from being removed
  if (s < (T)-1) out[blockIdx.x] = s;
}

template <typename T>
md_status time_chains(int sms, int iters, double* gflops) {
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * 64 * (size_t)sms) != cudaSuccess) return MD_OUT_OF_MEMORY;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = 8 * sms;  // 2048 threads per SM
  const T a = (T)0.999999, b = (T)1e-7;
  double best = 0.0;
  k_fma_chains<T><<<blocks, kThreads>>>(out, iters, a, b);  // warm-up (clocks up)
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0);
    k_fma_chains<T><<<blocks, kThreads>>>(out, iters, a, b);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double fmas = (double)blocks * kThreads * kChains * (double)iters;
    if (ms > 0.f) best = fmax(best, 2.0 * fmas / (ms * 1e-3) * 1e-9);
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return MD_CUDA_ERROR;
  *gflops = best;
  return MD_OK;
}

}  // namespace

extern "C" md_status md_measure_arith_peaks(int device, double* fp64_gflops,
                                            double* fp32_gflops) {
  if (!fp64_gflops || !fp32_gflops) return MD_BAD_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return MD_NO_DEVICE;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      sms <= 0)
    return MD_NO_DEVICE;
  // about 50 ms per FP64 launch and 10 ms per FP32 launch on a GB300
  md_status s = time_chains<double>(sms, 4096, fp64_gflops);
  if (s != MD_OK) return s;
  return time_chains<float>(sms, 65536, fp32_gflops);
}

extern "C" md_status md_device_sm_count(int device, int* sms) {
  if (!sms) return MD_BAD_ARGUMENT;
  if (cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return MD_NO_DEVICE;
  return MD_OK;
}
