// Animation frames and the many-body pair list on the device.
//
// Frames: the reference copies the state into float arrays on the host at
// every animation step (pushAnim, common/Results.cpp:12-31) and writes them
// at the end (writeAnimationBinaryData, :51-86).  Here the conversion runs
// as a kernel into a device slot; the engine streams the slot to pinned host
// memory on a copy stream, so an animation step costs the step loop one
// small kernel and no host round trip.
//
// Pairs: tailResults (common/Results.cpp:88-118) tests all i < j of the
// many-body atoms in FP64.  One thread per i walks the j > i in shared-memory
// tiles; an FP32 screen drops the pairs far beyond the threshold and the
// rest are decided with the reference's arithmetic (separate products and
// sums, correctly rounded sqrt, `dist < 2 * reNO` with reNO the float
// 1.15f).  A counting pass and a writing pass keep the reference's order.
#include <algorithm>
#include <vector>

#include "md_output.h"

namespace mdgb {
namespace {

__global__ void k_anim_pack(const md_double4* __restrict__ pos, const double* __restrict__ vel,
                            const int* __restrict__ orig, int n, float* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int i = orig ? orig[p] : p;
  const md_double4 r = pos[p];
  float4* op = (float4*)out;
  op[i] = make_float4((float)r.x, (float)r.y, (float)r.z, (float)r.w);
  float* ov = out + 4 * (size_t)n;
  ov[3 * (size_t)i] = (float)vel[3 * (size_t)p];
  ov[3 * (size_t)i + 1] = (float)vel[3 * (size_t)p + 1];
  ov[3 * (size_t)i + 2] = (float)vel[3 * (size_t)p + 2];
}

constexpr int kTailThreads = 256;
// (float)(2 * reNO) with reNO = 1.15f (common/Constants.h:25): the product is
// formed in float and compared after promotion to double
constexpr float kTwoReNO = 2 * 1.15f;

template <bool WRITE>
__global__ void __launch_bounds__(kTailThreads)
    k_tail(const md_double4* __restrict__ pos, int n, int* __restrict__ cnt,
           const int* __restrict__ off, int* __restrict__ pairs, int capacity) {
  __shared__ md_double4 tj[kTailThreads];
  __shared__ float4 tf[kTailThreads];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < n;
  md_double4 a = live ? pos[i] : pos[0];
  const float4 af = make_float4((float)a.x, (float)a.y, (float)a.z, 0.f);
  const int ta = (int)a.w;
  // screen: an FP32 squared distance 2% above (2 reNO)^2 cannot pass (the
  // FP32 coordinates are within 1e-7 relative of the FP64 ones)
  const float screen = (kTwoReNO * 1.01f) * (kTwoReNO * 1.01f);
  int found = 0;
  int o = (WRITE && live) ? off[i] : 0;
  const int j_first = blockIdx.x * blockDim.x;  // tiles start at the block's first i
  for (int j0 = j_first; j0 < n; j0 += kTailThreads) {
    __syncthreads();
    const int jl = j0 + threadIdx.x;
    if (jl < n) {
      const md_double4 b = pos[jl];
      tj[threadIdx.x] = b;
      tf[threadIdx.x] = make_float4((float)b.x, (float)b.y, (float)b.z, 0.f);
    }
    __syncthreads();
    if (!live) continue;
    const int jend = min(kTailThreads, n - j0);
    for (int k = 0; k < jend; k++) {
      const int j = j0 + k;
      if (j <= i) continue;
      const float4 bf = tf[k];
      const float fx = af.x - bf.x, fy = af.y - bf.y, fz = af.z - bf.z;
      if (fx * fx + fy * fy + fz * fz > screen) continue;
      const md_double4 b = tj[k];
      if ((int)b.w == ta) continue;
      const double dx = __dsub_rn(a.x, b.x), dy = __dsub_rn(a.y, b.y), dz = __dsub_rn(a.z, b.z);
      const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      if (__dsqrt_rn(d2) < (double)kTwoReNO) {
        if (WRITE) {
          if (o < capacity) {
            pairs[2 * (size_t)o] = i;
            pairs[2 * (size_t)o + 1] = j;
          }
          o++;
        }
        found++;
      }
    }
  }
  if (!WRITE && live) cnt[i] = found;
}

}  // namespace

void launch_anim_pack(const md_double4* pos, const double* vel, const int* orig, int n,
                      float* out, cudaStream_t st) {
  if (n <= 0) return;
  k_anim_pack<<<(n + 255) / 256, 256, 0, st>>>(pos, vel, orig, n, out);
}

int tail_pairs(const md_double4* pos, int n, int* pairs, int capacity, int* count,
               cudaStream_t st) {
  *count = 0;
  if (n < 2) return 0;
  int* cnt = nullptr;
  int* dpairs = nullptr;
  cudaError_t e = cudaMalloc(&cnt, sizeof(int) * 2 * (size_t)n);
  if (e != cudaSuccess) return (int)e;
  int* off = cnt + n;
  const int blocks = (n + kTailThreads - 1) / kTailThreads;
  k_tail<false><<<blocks, kTailThreads, 0, st>>>(pos, n, cnt, nullptr, nullptr, 0);
  std::vector<int> h(n);
  e = cudaMemcpyAsync(h.data(), cnt, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  long long total = 0;
  if (e == cudaSuccess) {
    for (int i = 0; i < n; i++) {
      const int c = h[i];
      h[i] = (int)std::min<long long>(total, 0x7fffffff);
      total += c;
    }
    *count = (int)std::min<long long>(total, 0x7fffffff);
  }
  const int keep = (int)std::min<long long>(total, capacity > 0 ? capacity : 0);
  if (e == cudaSuccess && keep > 0 && pairs) {
    e = cudaMalloc(&dpairs, sizeof(int) * 2 * (size_t)keep);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(off, h.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      k_tail<true><<<blocks, kTailThreads, 0, st>>>(pos, n, nullptr, off, dpairs, keep);
      e = cudaMemcpyAsync(pairs, dpairs, sizeof(int) * 2 * (size_t)keep, cudaMemcpyDeviceToHost,
                          st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (dpairs) cudaFree(dpairs);
  cudaFree(cnt);
  return (int)e;
}

}  // namespace mdgb
