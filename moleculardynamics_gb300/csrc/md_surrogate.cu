// Learned surrogate of the bond-order term (common/arvdwfc + the bond-order
// functions of cpu/common/BondOrderFuncs.h): per-atom Behler symmetry
// functions (16 radial, 16 angular, FP32), a 32-64-64-1 MLP with BF16
// weights on the tensor cores (tcgen05, FP32 accumulation in tensor memory),
// forces from the network's analytic gradient, Adam training on per-atom
// energies of the exact method, and the tensor-core self-test.
#include <cuda_bf16.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include <algorithm>

#include "../../include/mdgb.h"
#include "md_neighbor.cuh"
#include "md_surrogate.h"
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

// ---------------------------------------------------------------- surrogate
constexpr int kDesc = kSurDesc, kHid = 64, kRad = 16, kAng = 16;
constexpr int kSgMax = 64;  // neighbours within the descriptor cutoff
constexpr int oW1 = 0, oB1 = oW1 + kHid * kDesc, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid,
              oW3 = oB2 + kHid, oB3 = oW3 + kHid, kParams = oB3 + 1;  // 6337

DescParams default_desc(float rc) {
  DescParams P;
  P.rc = rc;
  const float d = (rc - 0.8f) / (kRad - 1);
  P.eta_r = 0.5f / (d * d);
  for (int k = 0; k < kRad; k++) P.rs[k] = 0.8f + d * k;
  // the kernels rely on this layout (ang_pair): f = 8 e + 4 l + z
  const int zetas[4] = {1, 2, 4, 16};
  const float etas[2] = {0.02f, 0.25f};
  for (int f = 0; f < kAng; f++) {
    P.zeta[f] = zetas[f % 4];
    P.lam[f] = (f / 4) % 2 ? -1.f : 1.f;
    P.eta_a[f] = etas[f / 8];
    P.pref[f] = powf(2.f, 1.f - (float)P.zeta[f]);
  }
  return P;
}

__device__ __forceinline__ void fcut(float r, float rc, float& fc, float& dfc) {
  const float a = 3.14159265358979f / rc;
  float s, c;
  __sincosf(a * r, &s, &c);
  fc = 0.5f * (c + 1.f);
  dfc = -0.5f * a * s;
}

// Angular factors of one neighbour pair for the 16 functions f = 8 e + 4 l + z
// of default_desc's table (eta index e, lambda index l for +1 / -1, zeta index
// z for 1, 2, 4, 16): powers of both bases by squaring and one exponential
// per eta, instead of 16 of each.
struct AngPair {
  float b[2];        // 1 + lambda cos
  float pz[2][4];    // b ^ zeta
  float pz1[2][4];   // b ^ (zeta - 1)
  float ex[2];       // exp(-eta q)
};

__device__ __forceinline__ void ang_pair(float c, float q, const DescParams& P, AngPair& A) {
#pragma unroll
  for (int l = 0; l < 2; l++) {
    const float b = l ? 1.f - c : 1.f + c;
    const float p2 = b * b, p4 = p2 * p2, p8 = p4 * p4;
    A.b[l] = b;
    A.pz[l][0] = b;
    A.pz[l][1] = p2;
    A.pz[l][2] = p4;
    A.pz[l][3] = p8 * p8;
    A.pz1[l][0] = 1.f;
    A.pz1[l][1] = b;
    A.pz1[l][2] = p2 * b;
    A.pz1[l][3] = p8 * p4 * p2 * b;
  }
  A.ex[0] = __expf(-P.eta_a[0] * q);
  A.ex[1] = __expf(-P.eta_a[8] * q);
}

// neighbours of i within rc (from the bond-order candidate rows: the 27
// build-time cells around i, as walk_row visits them), as packed entries
// with their periodic image; one warp per atom, lanes over the cells' atoms
// joined into one list, kept entries compacted in candidate order with a ballot
// (distances in FP32 from an FP32 copy of the positions: a neighbour at the
// cutoff enters the descriptors with weight fc(rc) = 0 either way)
__global__ void __launch_bounds__(128)
    k_sg_short(const float4* __restrict__ pos, RowWalker w, float rc,
               uint32_t* __restrict__ sl, int* __restrict__ slen, int* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (i >= w.n) return;  // whole warp
  const float4 pi = pos[i];
  const float rc2 = rc * rc;
  const float boxf = (float)w.g.box;
  const int4 c4 = reinterpret_cast<const int4*>(w.cell3)[i];
  const int cx = c4.x, cy = c4.y, cz = c4.z;
  const int cells = w.g.cells;
  // lane c < 27 looks up cell c of the 27 (dx slowest, dz fastest) with its image
  int cs = 0, cn = 0, im[3] = {0, 0, 0};
  if (lane < 27) {
    int nc[3] = {cx + lane / 9 - 1, cy + (lane / 3) % 3 - 1, cz + lane % 3 - 1};
    bool out = false;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      if (!w.g.periodic) {
        if (nc[d] >= cells || nc[d] < 0) out = true;
      } else {
        if (nc[d] < 0) { nc[d] += cells; im[d] = -1; }
        if (nc[d] >= cells) { nc[d] -= cells; im[d] = 1; }
      }
    }
    if (!out) {
      const int slot = table_find(w.keys, w.cap, cell_key(nc[0], nc[1], nc[2]));
      if (slot >= 0) {
        cs = w.start[slot];
        cn = w.count[slot];
      }
    }
  }
  // the cells' atoms as one list in cell order: inclusive prefix of the counts
  int incl = cn;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const int excl = incl - cn;
  int cnt = 0;
  for (int v0 = 0; v0 < total; v0 += 32) {
    const int v = v0 + lane;
    // cell of candidate v: the first c with incl_c > v (27 cells: five halvings)
    int lo = 0, hi = 26;
#pragma unroll
    for (int it = 0; it < 5; it++) {
      const int mid = (lo + hi) >> 1;
      if (__shfl_sync(0xffffffffu, incl, mid) > v)
        hi = mid;
      else
        lo = mid + 1;
    }
    const int c = min(lo, 26);
    const int base = __shfl_sync(0xffffffffu, cs, c) - __shfl_sync(0xffffffffu, excl, c);
    const int ix = __shfl_sync(0xffffffffu, im[0], c), iy = __shfl_sync(0xffffffffu, im[1], c),
              iz = __shfl_sync(0xffffffffu, im[2], c);
    bool keep = false;
    int m = 0;
    if (v < total) {
      m = w.sorted[base + v];
      if (m != i) {
        const float4 pm = pos[m];
        const float ddx = fmaf((float)ix, boxf, pm.x) - pi.x;
        const float ddy = fmaf((float)iy, boxf, pm.y) - pi.y;
        const float ddz = fmaf((float)iz, boxf, pm.z) - pi.z;
        keep = ddx * ddx + ddy * ddy + ddz * ddz < rc2;
      }
    }
    const unsigned mask = __ballot_sync(0xffffffffu, keep);
    const int at = cnt + __popc(mask & ((1u << lane) - 1u));
    if (keep && at < kSgMax) sl[(size_t)i * kSgMax + at] = pack_entry(m, ix, iy, iz);
    cnt += __popc(mask);
  }
  if (lane == 0) {
    if (cnt > kSgMax) atomicOr(status, ST_CELL_OVERFLOW);
    slen[i] = cnt < kSgMax ? cnt : kSgMax;
  }
}

// ---- warp-per-atom descriptor and force kernels (4 atoms per block) ----
struct NbrSm {
  float dx[kSgMax], dy[kSgMax], dz[kSgMax], r[kSgMax], ir[kSgMax], fc[kSgMax], dfc[kSgMax];
  int idx[kSgMax];
};

// neighbours of atom i into the warp's shared arrays; returns their count
__device__ __forceinline__ int warp_load_nbrs(int i, const md_double4* pos, const uint32_t* sl,
                                              const int* slen, double box, float rc,
                                              NbrSm& N) {
  const int lane = threadIdx.x & 31;
  const md_double4 pi = pos[i];
  const int S = slen[i];
  for (int s = lane; s < S; s += 32) {
    const uint32_t e = sl[(size_t)i * kSgMax + s];
    const int j = entry_index(e);
    const md_double4 pj = pos[j];
    const float dx = (float)(pj.x + entry_img(e, 0) * box - pi.x);
    const float dy = (float)(pj.y + entry_img(e, 1) * box - pi.y);
    const float dz = (float)(pj.z + entry_img(e, 2) * box - pi.z);
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    float fc, dfc;
    fcut(r, rc, fc, dfc);
    N.dx[s] = dx;
    N.dy[s] = dy;
    N.dz[s] = dz;
    N.r[s] = r;
    N.ir[s] = 1.f / r;  // the pair terms multiply by it instead of dividing
    N.fc[s] = fc;
    N.dfc[s] = dfc;
    N.idx[s] = j;
  }
  __syncwarp();
  return S;
}

// k-th pair (a < b) of S neighbours in row-major order
__device__ __forceinline__ void pair_of(int k, int S, int& a, int& b) {
  const int m = 2 * S - 1;
  int aa = (int)(0.5f * ((float)m - sqrtf((float)(m * m - 8 * k))));
  aa = max(0, min(aa, S - 2));
  auto off = [&](int x) { return x * (2 * S - x - 1) / 2; };
  while (aa > 0 && off(aa) > k) aa--;
  while (aa + 1 <= S - 2 && off(aa + 1) <= k) aa++;
  a = aa;
  b = k - off(aa) + aa + 1;
}

// k-th pair (a < b) of S neighbours in diagonal order: pairs (a, a + d) for
// d = 1, 2, ... in turn, so consecutive k have distinct a and distinct b
// (lanes of a warp update distinct neighbours' force sums)
__device__ __forceinline__ void pair_of_diag(int k, int S, int& a, int& b) {
  // offset of diagonal d: (d - 1) S - (d - 1) d / 2
  auto off = [&](int d) { return (d - 1) * S - (d - 1) * d / 2; };
  const float m = (float)(2 * S - 1);
  int d = 1 + (int)(0.5f * (m - sqrtf(fmaxf(m * m - 8.f * (float)k, 0.f))));
  d = max(1, min(d, S - 1));
  while (d > 1 && off(d) > k) d--;
  while (d + 1 <= S - 1 && off(d + 1) <= k) d++;
  a = k - off(d);
  b = a + d;
}

// sum over the warp of 32 per-lane vectors: lane f ends with component f
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16, h = 16; o > 0; o >>= 1, h >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < h; k++) {
      const float send = up ? v[k] : v[k + h];
      const float keep = up ? v[k + h] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return v[0];
}

// descriptors of atom i (one warp); out: normalised (G - mean) * istd, or raw G
__global__ void __launch_bounds__(128)
    k_sg_desc(const md_double4* __restrict__ pos, int n, const uint32_t* __restrict__ sl,
              const int* __restrict__ slen, double box, DescParams P,
              const float* __restrict__ mean, const float* __restrict__ istd,
              float* __restrict__ out) {
  __shared__ NbrSm nb[4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 4 + warp;
  if (i >= n) return;  // whole warp
  NbrSm& N = nb[warp];
  const int S = warp_load_nbrs(i, pos, sl, slen, box, P.rc, N);
  float v[32];
#pragma unroll
  for (int f = 0; f < 32; f++) v[f] = 0.f;
  for (int s = lane; s < S; s += 32) {
#pragma unroll
    for (int k = 0; k < kRad; k++) {
      const float t = N.r[s] - P.rs[k];
      v[k] += __expf(-P.eta_r * t * t) * N.fc[s];
    }
  }
  const int npair = S * (S - 1) / 2;
  for (int k = lane; k < npair; k += 32) {
    int a, b;
    pair_of(k, S, a, b);
    const float c = (N.dx[a] * N.dx[b] + N.dy[a] * N.dy[b] + N.dz[a] * N.dz[b]) * (N.ir[a] * N.ir[b]);
    const float q = N.r[a] * N.r[a] + N.r[b] * N.r[b];
    const float ff = N.fc[a] * N.fc[b];
    AngPair T;
    ang_pair(c, q, P, T);
#pragma unroll
    for (int f = 0; f < kAng; f++) {
      const int e = f >> 3, l = (f >> 2) & 1, z = f & 3;
      const float pz = T.b[l] > 0.f ? T.pz[l][z] : 0.f;
      v[kRad + f] += P.pref[f] * pz * T.ex[e] * ff;
    }
  }
  const float G = warp_reduce_scatter32(v);
  out[(size_t)i * kDesc + lane] = mean ? (G - mean[lane]) * istd[lane] : G;
}

// forces from g_if = dE_i/dG_if (one warp per atom i; neighbour forces
// gathered in shared memory, then one global atomic per neighbour)
__global__ void __launch_bounds__(128)
    k_sg_force(const md_double4* __restrict__ pos, int n, const uint32_t* __restrict__ sl,
               const int* __restrict__ slen, double box, DescParams P,
               const float* __restrict__ gcoef, float* __restrict__ F32) {
  __shared__ NbrSm nb[4];
  __shared__ float fn[4][3][kSgMax];
  __shared__ float gs[4][kDesc];
  __shared__ float gz[4][kAng];  // g_f pref_f zeta_f lambda_f of the angular functions
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 4 + warp;
  if (i >= n) return;  // whole warp
  NbrSm& N = nb[warp];
  {
    const float gv = gcoef[(size_t)i * kDesc + lane];
    // angular coefficients carry their prefactor 2^(1 - zeta)
    const int f = lane - kRad;
    gs[warp][lane] = f >= 0 ? gv * P.pref[f] : gv;
    if (f >= 0) gz[warp][f] = gv * P.pref[f] * (float)P.zeta[f] * P.lam[f];
  }
  for (int s = lane; s < kSgMax; s += 32) fn[warp][0][s] = fn[warp][1][s] = fn[warp][2][s] = 0.f;
  const int S = warp_load_nbrs(i, pos, sl, slen, box, P.rc, N);  // ends with __syncwarp
  const float* g = gs[warp];
  float fix = 0.f, fiy = 0.f, fiz = 0.f;
  for (int s = lane; s < S; s += 32) {
    float sum = 0.f;  // sum_k g_k dphi_k/dr
#pragma unroll
    for (int k = 0; k < kRad; k++) {
      const float t = N.r[s] - P.rs[k];
      sum += g[k] * __expf(-P.eta_r * t * t) * (-2.f * P.eta_r * t * N.fc[s] + N.dfc[s]);
    }
    const float ir = N.ir[s];
    const float gx = sum * N.dx[s] * ir, gy = sum * N.dy[s] * ir, gz = sum * N.dz[s] * ir;
    // dG/dr_j = +grad, dG/dr_i = -grad; F = -dE/dr
    fn[warp][0][s] -= gx;
    fn[warp][1][s] -= gy;
    fn[warp][2][s] -= gz;
    fix += gx;
    fiy += gy;
    fiz += gz;
  }
  __syncwarp();
  const float* gzw = gz[warp];
  const int npair = S * (S - 1) / 2;
  for (int k = lane; k < npair; k += 32) {
    int a, b;
    pair_of_diag(k, S, a, b);
    const float ra = N.r[a], rb = N.r[b];
    const float ia = N.ir[a], ib = N.ir[b], irab = ia * ib;
    const float c = (N.dx[a] * N.dx[b] + N.dy[a] * N.dy[b] + N.dz[a] * N.dz[b]) * irab;
    const float q = ra * ra + rb * rb;
    const float fca = N.fc[a], fcb = N.fc[b], dfa = N.dfc[a], dfb = N.dfc[b];
    AngPair T;
    ang_pair(c, q, P, T);
    // the sums over f = 8 e + 4 l + z factor per eta index e:
    //   A  = fca fcb sum_e ex_e sum_lz g' zeta lambda b^(zeta-1)
    //   Ba = fcb sum_e ex_e (-2 eta_e ra fca + dfa) sum_lz g' b^zeta, Bb likewise
    float A = 0.f, Ba = 0.f, Bb = 0.f;
#pragma unroll
    for (int e = 0; e < 2; e++) {
      float se = 0.f, ae = 0.f;
#pragma unroll
      for (int l = 0; l < 2; l++) {
        const float on = T.b[l] > 0.f ? 1.f : 0.f;  // (1 + lambda cos) clipped at 0
#pragma unroll
        for (int z = 0; z < 4; z++) {
          const int f = 8 * e + 4 * l + z;
          se = fmaf(on * g[kRad + f], T.pz[l][z], se);
          ae = fmaf(on * gzw[f], T.pz1[l][z], ae);
        }
      }
      const float eta = P.eta_a[8 * e];
      A = fmaf(ae, T.ex[e], A);
      se *= T.ex[e];
      Ba = fmaf(se, fmaf(-2.f * eta * ra, fca, dfa), Ba);
      Bb = fmaf(se, fmaf(-2.f * eta * rb, fcb, dfb), Bb);
    }
    A *= fca * fcb;
    Ba *= fcb;
    Bb *= fca;
    // dc/dd_a = d_b / (ra rb) - c d_a / ra^2
    const float gax = A * (N.dx[b] * irab - c * N.dx[a] * ia * ia) + Ba * N.dx[a] * ia;
    const float gay = A * (N.dy[b] * irab - c * N.dy[a] * ia * ia) + Ba * N.dy[a] * ia;
    const float gaz = A * (N.dz[b] * irab - c * N.dz[a] * ia * ia) + Ba * N.dz[a] * ia;
    const float gbx = A * (N.dx[a] * irab - c * N.dx[b] * ib * ib) + Bb * N.dx[b] * ib;
    const float gby = A * (N.dy[a] * irab - c * N.dy[b] * ib * ib) + Bb * N.dy[b] * ib;
    const float gbz = A * (N.dz[a] * irab - c * N.dz[b] * ib * ib) + Bb * N.dz[b] * ib;
    atomicAdd(&fn[warp][0][a], -gax);
    atomicAdd(&fn[warp][1][a], -gay);
    atomicAdd(&fn[warp][2][a], -gaz);
    atomicAdd(&fn[warp][0][b], -gbx);
    atomicAdd(&fn[warp][1][b], -gby);
    atomicAdd(&fn[warp][2][b], -gbz);
    fix += gax + gbx;
    fiy += gay + gby;
    fiz += gaz + gbz;
  }
  __syncwarp();
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fix += __shfl_xor_sync(0xffffffffu, fix, o);
    fiy += __shfl_xor_sync(0xffffffffu, fiy, o);
    fiz += __shfl_xor_sync(0xffffffffu, fiz, o);
  }
  for (int s = lane; s < S; s += 32) {
    atomicAdd(&F32[3 * N.idx[s]], fn[warp][0][s]);
    atomicAdd(&F32[3 * N.idx[s] + 1], fn[warp][1][s]);
    atomicAdd(&F32[3 * N.idx[s] + 2], fn[warp][2][s]);
  }
  if (lane == 0) {
    atomicAdd(&F32[3 * i], fix);
    atomicAdd(&F32[3 * i + 1], fiy);
    atomicAdd(&F32[3 * i + 2], fiz);
  }
}

__global__ void k_sg_pos32(const md_double4* __restrict__ pos, int n, float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const md_double4 p = pos[i];
  out[i] = make_float4((float)p.x, (float)p.y, (float)p.z, 0.f);
}

// skip (optional, device): when set, the forces are not stored and
// skipped (device, optional) counts the call once
__global__ void k_sg_store(const float* __restrict__ F32, double* __restrict__ f3, int n,
                           int accumulate, const int* __restrict__ skip,
                           int* __restrict__ skipped) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (skip && *skip) {
    if (k == 0 && skipped) atomicAdd(skipped, 1);
    return;
  }
  if (k >= 3 * n) return;
  f3[k] = accumulate ? f3[k] + (double)F32[k] : (double)F32[k];
}

// ---- the network: 32 -> 64 (tanh) -> 64 (tanh) -> 1, BF16 weights ----
// Device weight copies for the tensor cores, K-major B operands:
// W1 [64 out][32 in], W1T [32 in][64 out], W2 [64 out][64 in], W2T [64 in][64 out].
struct NetDev {
  const __nv_bfloat16 *W1, *W1T, *W2, *W2T;
  const float* P;  // FP32 master parameters (biases and w3 used from here)
};

// shared-memory plan of the network kernels (bytes)
constexpr int kSmA = 0;                  // 128 x 64 BF16 operand (16 KB)
constexpr int kSmB = kSmA + 16384;       // 128 x 64 BF16 operand (16 KB)
constexpr int kSmW1 = kSmB + 16384;      // 64 x 32 (4 KB)
constexpr int kSmW1T = kSmW1 + 4096;     // 32 x 64 (4 KB)
constexpr int kSmW2 = kSmW1T + 4096;     // 64 x 64 (8 KB)
constexpr int kSmW2T = kSmW2 + 8192;     // 64 x 64 (8 KB)
constexpr int kSmAT = kSmW2T + 8192;     // training: 128 x 128 BF16 (32 KB)
constexpr int kSmBT = kSmAT + 32768;     // training: 64 x 128 BF16 (16 KB)
constexpr int kSmTrain = kSmBT + 16384;  // 104 KB
constexpr int kSmALo = kSmAT;            // inference: low BF16 parts of A / B operands
constexpr int kSmBLo = kSmALo + 16384;
constexpr int kSmInfer = kSmBLo + 16384; // 88 KB

__device__ __forceinline__ void put_bf16(unsigned char* base, int r, int k, int K, float v) {
  *(__nv_bfloat16*)(base + tc_offset(r, k, K)) = __float2bfloat16_rn(v);
}

// weights (row-major BF16 R x K in global) into the K-major tile layout
__device__ __forceinline__ void load_tile(unsigned char* dst, const __nv_bfloat16* src, int R,
                                          int K) {
  for (int e = threadIdx.x; e < R * K; e += blockDim.x)
    *(__nv_bfloat16*)(dst + tc_offset(e / K, e % K, K)) = src[e];
}

// a value as the sum of two BF16 numbers (hi = round(v), lo = round(v - hi)):
// products of hi and lo parts with BF16 weights keep the network input and
// hidden activations to about 16 significant bits, so the energy is a smooth
// function of the positions and the forces are its gradient
__device__ __forceinline__ void put_split(unsigned char* hi, unsigned char* lo, int r, int k,
                                          int K, float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  *(__nv_bfloat16*)(hi + tc_offset(r, k, K)) = h;
  *(__nv_bfloat16*)(lo + tc_offset(r, k, K)) = __float2bfloat16_rn(v - __bfloat162float(h));
}

// operands written by threads -> visible to the tensor core; then one thread
// issues the product (A + Alo when given) and all wait for its completion
__device__ __forceinline__ bool tc_run(uint32_t d, const unsigned char* A, const unsigned char* B,
                                       int N, int K, uint64_t* bar, uint32_t& phase,
                                       int* status, const unsigned char* Alo = nullptr) {
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x == 0) {
    if (Alo) {
      tc_gemm_issue(d, A, B, N, K, nullptr);
      tc_gemm_issue(d, Alo, B, N, K, bar, true);
    } else {
      tc_gemm_issue(d, A, B, N, K, bar);
    }
  }
  const bool ok = mbar_wait(bar, phase, status);
  phase ^= 1u;
  tc_fence_after();
  return __syncthreads_and(ok);
}

__device__ __forceinline__ float tanh_fast(float x) {
  // tanh(x) = 1 - 2 / (exp(2x) + 1)
  return 1.f - 2.f / (__expf(2.f * x) + 1.f);
}

// Inference on 128 atoms per CTA: t_i = net(x_i) and dt/dx_i (4 tensor-core
// products: two forward, two for the input gradient; every A operand as a
// pair of BF16 parts).
__global__ void __launch_bounds__(128, 1)
    k_net_infer(const float* __restrict__ X, int n, NetDev w, float* __restrict__ t_out,
                float* __restrict__ dtdx, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_taddr;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = 32 * warp + (tid & 31);
  const int i = blockIdx.x * 128 + row;
  const bool live = i < n;
  unsigned char* A = sm + kSmA;
  unsigned char* B = sm + kSmB;
  unsigned char* Al = sm + kSmALo;
  unsigned char* Bl = sm + kSmBLo;
  load_tile(sm + kSmW1, w.W1, kHid, kDesc);
  load_tile(sm + kSmW1T, w.W1T, kDesc, kHid);
  load_tile(sm + kSmW2, w.W2, kHid, kHid);
  load_tile(sm + kSmW2T, w.W2T, kHid, kHid);
  for (int f = 0; f < kDesc; f++)
    put_split(A, Al, row, f, kDesc, live ? X[(size_t)i * kDesc + f] : 0.f);
  if (warp == 0) tc_alloc(&s_taddr, 128);
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = s_taddr + ((uint32_t)(32 * warp) << 16);
  uint32_t phase = 0;
  bool ok = tc_run(s_taddr, A, sm + kSmW1, kHid, kDesc, &bar, phase, status, Al);
  float h1[kHid];
  if (ok) {
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float v[16];
      tc_ld16(tm + c0, v);
#pragma unroll
      for (int k = 0; k < 16; k++) {
        h1[c0 + k] = tanh_fast(v[k] + w.P[oB1 + c0 + k]);
        put_split(B, Bl, row, c0 + k, kHid, h1[c0 + k]);
      }
    }
    ok = tc_run(s_taddr + 64, B, sm + kSmW2, kHid, kHid, &bar, phase, status, Bl);
  }
  if (ok) {
    float t = w.P[oB3];
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float v[16];
      tc_ld16(tm + 64 + c0, v);
#pragma unroll
      for (int k = 0; k < 16; k++) {
        const float h2 = tanh_fast(v[k] + w.P[oB2 + c0 + k]);
        const float w3 = w.P[oW3 + c0 + k];
        t = fmaf(w3, h2, t);
        put_split(A, Al, row, c0 + k, kHid, w3 * (1.f - h2 * h2));  // delta2
      }
    }
    if (live) t_out[i] = t;
    ok = tc_run(s_taddr, A, sm + kSmW2T, kHid, kHid, &bar, phase, status, Al);
  }
  if (ok) {
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float v[16];
      tc_ld16(tm + c0, v);
#pragma unroll
      for (int k = 0; k < 16; k++)
        put_split(B, Bl, row, c0 + k, kHid, v[k] * (1.f - h1[c0 + k] * h1[c0 + k]));  // delta1
    }
    ok = tc_run(s_taddr + 64, B, sm + kSmW1T, kDesc, kHid, &bar, phase, status, Bl);
  }
  if (ok) {  // every lane reads (tcgen05.ld is warp-collective); live rows store
    for (int c0 = 0; c0 < kDesc; c0 += 16) {
      float v[16];
      tc_ld16(tm + 64 + c0, v);
      if (live) {
#pragma unroll
        for (int k = 0; k < 16; k++) dtdx[(size_t)i * kDesc + c0 + k] = v[k];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(s_taddr, 128);
}

// 64-bit mix of (seed, k) for batch sampling
__device__ __forceinline__ unsigned long long mix2(unsigned long long a, unsigned long long b) {
  unsigned long long z = a * 0x9E3779B97F4A7C15ULL + b + 0x632BE59BD9B4E019ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float col_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One training pass over 128 samples per CTA: forward, squared loss on the
// normalised per-atom energy, backward; gradients are accumulated into grad
// (FP32, same layout as the parameters) and loss into loss[0].
// Samples: rows sel(k) of X/T, sel = explicit list, or hashed from seed.
__global__ void __launch_bounds__(128, 1)
    k_net_train(const float* __restrict__ X, const float* __restrict__ T, int nsamples,
                const int* __restrict__ rows, int nrows, unsigned long long seed, NetDev w,
                float inv_batch, float* __restrict__ grad, double* __restrict__ loss,
                int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_taddr;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = 32 * warp + lane;
  const int k = blockIdx.x * 128 + row;
  const bool live = k < nrows;
  int src = 0;
  if (live) src = rows ? rows[k] : (int)(mix2(seed, (unsigned long long)k) % (unsigned long long)nsamples);
  unsigned char* A = sm + kSmA;
  unsigned char* B = sm + kSmB;
  unsigned char* AT = sm + kSmAT;
  unsigned char* BT = sm + kSmBT;
  load_tile(sm + kSmW1, w.W1, kHid, kDesc);
  load_tile(sm + kSmW2, w.W2, kHid, kHid);
  load_tile(sm + kSmW2T, w.W2T, kHid, kHid);
  for (int e = tid; e < 32768 / 16; e += blockDim.x) ((uint4*)AT)[e] = make_uint4(0, 0, 0, 0);
  float x[kDesc];
  for (int f = 0; f < kDesc; f++) {
    x[f] = live ? X[(size_t)src * kDesc + f] : 0.f;
    put_bf16(A, row, f, kDesc, x[f]);
  }
  if (warp == 0) tc_alloc(&s_taddr, 256);
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = s_taddr + ((uint32_t)(32 * warp) << 16);
  uint32_t phase = 0;
  float h1[kHid];
  bool ok = tc_run(s_taddr, A, sm + kSmW1, kHid, kDesc, &bar, phase, status);
  if (ok) {
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float v[16];
      tc_ld16(tm + c0, v);
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int c = c0 + q;
        h1[c] = tanh_fast(v[q] + w.P[oB1 + c]);
        put_bf16(B, row, c, kHid, h1[c]);
        put_bf16(BT, c, row, 128, h1[c]);  // H1^T: B operand of the W2 gradient
      }
    }
    ok = tc_run(s_taddr + 64, B, sm + kSmW2, kHid, kHid, &bar, phase, status);
  }
  float d3 = 0.f;
  if (ok) {
    float h2[kHid];
    float t = w.P[oB3];
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float v[16];
      tc_ld16(tm + 64 + c0, v);
#pragma unroll
      for (int q = 0; q < 16; q++) {
        h2[c0 + q] = tanh_fast(v[q] + w.P[oB2 + c0 + q]);
        t = fmaf(w.P[oW3 + c0 + q], h2[c0 + q], t);
      }
    }
    const float res = live ? t - T[src] : 0.f;
    d3 = 2.f * res * inv_batch;
    const double l = (double)res * res * inv_batch;
    const double lw = (double)col_sum((float)l);
    if (lane == 0) atomicAdd(loss, lw);
    const float gb3 = col_sum(d3);
    if (lane == 0) atomicAdd(&grad[oB3], gb3);
    for (int c = 0; c < kHid; c++) {
      const float gw3 = col_sum(d3 * h2[c]);
      const float d2 = d3 * w.P[oW3 + c] * (1.f - h2[c] * h2[c]);
      const float gb2 = col_sum(d2);
      if (lane == 0) {
        atomicAdd(&grad[oW3 + c], gw3);
        atomicAdd(&grad[oB2 + c], gb2);
      }
      put_bf16(A, row, c, kHid, d2);   // delta2 for dH1 = delta2 W2
      put_bf16(AT, c, row, 128, d2);   // delta2^T for the W2 gradient
    }
    // W2 gradient (rows out, cols in) and dH1, one commit for both
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      const uint32_t a0 = smem_addr(AT), b0 = smem_addr(BT);
      const uint32_t idesc = tc_idesc_bf16(128, kHid);
      for (int j = 0; j < 128 / 16; j++)
        tc_mma(s_taddr + 128, tc_desc(a0 + j * 256u, 128u, 128u * 16u),
               tc_desc(b0 + j * 256u, 128u, 128u * 16u), idesc, j > 0);
      const uint32_t a1 = smem_addr(A), b1 = smem_addr(sm + kSmW2T);
      for (int j = 0; j < kHid / 16; j++)
        tc_mma(s_taddr, tc_desc(a1 + j * 256u, 128u, kHid * 16u),
               tc_desc(b1 + j * 256u, 128u, kHid * 16u), idesc, j > 0);
      tc_commit(&bar);
    }
    const bool got = mbar_wait(&bar, phase, status);
    phase ^= 1u;
    tc_fence_after();
    ok = __syncthreads_and(got);
  }
  if (ok) {
    if (warp < 2) {  // rows 0..63 of the W2 gradient
      for (int c0 = 0; c0 < kHid; c0 += 16) {
        float v[16];
        tc_ld16(tm + 128 + c0, v);
#pragma unroll
        for (int q = 0; q < 16; q++) atomicAdd(&grad[oW2 + row * kHid + c0 + q], v[q]);
      }
    }
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float v[16];
      tc_ld16(tm + c0, v);
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int c = c0 + q;
        const float d1 = v[q] * (1.f - h1[c] * h1[c]);
        const float gb1 = col_sum(d1);
        if (lane == 0) atomicAdd(&grad[oB1 + c], gb1);
        put_bf16(AT, c, row, 128, d1);  // delta1^T
      }
    }
    for (int f = 0; f < kDesc; f++) put_bf16(BT, f, row, 128, x[f]);  // X^T
    ok = tc_run(s_taddr + 192, AT, BT, kDesc, 128, &bar, phase, status);
  }
  if (ok && warp < 2) {  // rows 0..63 of the W1 gradient
    for (int c0 = 0; c0 < kDesc; c0 += 16) {
      float v[16];
      tc_ld16(tm + 192 + c0, v);
#pragma unroll
      for (int q = 0; q < 16; q++) atomicAdd(&grad[oW1 + row * kDesc + c0 + q], v[q]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(s_taddr, 256);
}

// q_if = sum_j (e_j - e_i) . dG_if/dd_j for the force residual e (n x 3),
// written as v_if = scale * istd_f * q_if (the loss' sensitivity to dt/dx;
// istd NULL: 1).  One warp per atom as k_sg_desc: lanes over neighbours,
// then over neighbour pairs, each lane summing all 32 components, one
// reduce-scatter at the end.  Per pair the 16 angular terms share
//   K1 = fc_a fc_b (dc/dd_a . de_a + dc/dd_b . de_b) and, per eta index e,
//   K2_e = fc_b (-2 eta_e r_a fc_a + dfc_a) u_a + fc_a (-2 eta_e r_b fc_b + dfc_b) u_b,
// so q_f += pref_f ex_e (zeta_f lambda_f b^(zeta-1) K1 + b^zeta K2_e).
__global__ void __launch_bounds__(128)
    k_sg_ctrans(const md_double4* __restrict__ pos, int n, const uint32_t* __restrict__ sl,
                const int* __restrict__ slen, double box, DescParams P,
                const float* __restrict__ e3, float scale, const float* __restrict__ istd,
                float* __restrict__ V) {
  __shared__ NbrSm nb[4];
  __shared__ float dex[4][kSgMax], dey[4][kSgMax], dez[4][kSgMax];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 4 + warp;
  if (i >= n) return;  // whole warp
  NbrSm& N = nb[warp];
  const int S = warp_load_nbrs(i, pos, sl, slen, box, P.rc, N);  // ends with __syncwarp
  const float eix = e3[3 * i], eiy = e3[3 * i + 1], eiz = e3[3 * i + 2];
  float v[32];
#pragma unroll
  for (int f = 0; f < 32; f++) v[f] = 0.f;
  for (int s = lane; s < S; s += 32) {
    const int j = N.idx[s];
    const float ex = e3[3 * j] - eix, ey = e3[3 * j + 1] - eiy, ez = e3[3 * j + 2] - eiz;
    dex[warp][s] = ex;
    dey[warp][s] = ey;
    dez[warp][s] = ez;
    const float ud = (N.dx[s] * ex + N.dy[s] * ey + N.dz[s] * ez) * N.ir[s];  // u . de
#pragma unroll
    for (int k = 0; k < kRad; k++) {
      const float t = N.r[s] - P.rs[k];
      v[k] += __expf(-P.eta_r * t * t) * (-2.f * P.eta_r * t * N.fc[s] + N.dfc[s]) * ud;
    }
  }
  __syncwarp();
  const int npair = S * (S - 1) / 2;
  for (int k = lane; k < npair; k += 32) {
    int a, b;
    pair_of(k, S, a, b);
    const float ra = N.r[a], rb = N.r[b];
    const float ia = N.ir[a], ib = N.ir[b], irab = ia * ib;
    const float dax = N.dx[a], day = N.dy[a], daz = N.dz[a];
    const float dbx = N.dx[b], dby = N.dy[b], dbz = N.dz[b];
    const float eax = dex[warp][a], eay = dey[warp][a], eaz = dez[warp][a];
    const float ebx = dex[warp][b], eby = dey[warp][b], ebz = dez[warp][b];
    const float c = (dax * dbx + day * dby + daz * dbz) * irab;
    const float q2 = ra * ra + rb * rb;
    const float pa = dax * eax + day * eay + daz * eaz;  // d_a . de_a
    const float pb = dbx * ebx + dby * eby + dbz * ebz;
    const float dca = (dbx * eax + dby * eay + dbz * eaz) * irab - c * pa * ia * ia;
    const float dcb = (dax * ebx + day * eby + daz * ebz) * irab - c * pb * ib * ib;
    const float ua = pa * ia, ub = pb * ib;
    const float fca = N.fc[a], fcb = N.fc[b], dfa = N.dfc[a], dfb = N.dfc[b];
    AngPair T;
    ang_pair(c, q2, P, T);
    const float K1 = fca * fcb * (dca + dcb);
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const float eta = P.eta_a[8 * e];
      const float K2 = fcb * fmaf(-2.f * eta * ra, fca, dfa) * ua +
                       fca * fmaf(-2.f * eta * rb, fcb, dfb) * ub;
#pragma unroll
      for (int l = 0; l < 2; l++) {
        const float on = T.b[l] > 0.f ? T.ex[e] : 0.f;  // (1 + lambda cos) clipped at 0
#pragma unroll
        for (int z = 0; z < 4; z++) {
          const int f = 8 * e + 4 * l + z;
          const float zl = (float)P.zeta[f] * P.lam[f];
          v[kRad + f] += P.pref[f] * on * fmaf(zl * T.pz1[l][z], K1, T.pz[l][z] * K2);
        }
      }
    }
  }
  const float q = warp_reduce_scatter32(v);
  V[(size_t)i * kDesc + lane] = scale * (istd ? istd[lane] : 1.f) * q;
}

// e = F_pred - F_exact (FP32) and sum e^2 into acc[0]
__global__ void k_fm_resid(const float* __restrict__ F32, const double* __restrict__ fx, int n3,
                           float* __restrict__ e3, double* __restrict__ acc) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (k < n3) {
    const float e = F32[k] - (float)fx[k];
    e3[k] = e;
    s = (double)e * e;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(acc, s);
}

// shared-memory plan of the force-term training kernel (bytes)
constexpr int kFA = 0, kFA2 = 16384, kFB = 32768, kFB2 = 49152;
constexpr int kFW1 = 65536, kFW2 = kFW1 + 4096, kFW2T = kFW2 + 8192;
constexpr int kFAT = kFW2T + 8192, kFAT2 = kFAT + 32768;
constexpr int kFBT = kFAT2 + 32768, kFBT2 = kFBT + 16384;
constexpr int kSmForce = kFBT2 + 16384;  // 180 KB

// Parameter gradient of sum_i v_i . dt/dx(x_i) (the force-matching term),
// accumulated into grad: the network's tangent along v (forward) and the
// adjoint of that tangent, eight tensor-core products per 128 rows.
__global__ void __launch_bounds__(128, 1)
    k_net_train_force(const float* __restrict__ X, const float* __restrict__ V, int n, NetDev w,
                      float* __restrict__ grad, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_taddr;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = 32 * warp + lane;
  const int i = blockIdx.x * 128 + row;
  const bool live = i < n;
  unsigned char *A = sm + kFA, *A2 = sm + kFA2, *B = sm + kFB, *B2 = sm + kFB2;
  unsigned char *AT = sm + kFAT, *AT2 = sm + kFAT2, *BT = sm + kFBT, *BT2 = sm + kFBT2;
  load_tile(sm + kFW1, w.W1, kHid, kDesc);
  load_tile(sm + kFW2, w.W2, kHid, kHid);
  load_tile(sm + kFW2T, w.W2T, kHid, kHid);
  for (int e = tid; e < 2 * 32768 / 16; e += blockDim.x) ((uint4*)AT)[e] = make_uint4(0, 0, 0, 0);
  for (int f = 0; f < kDesc; f++) {
    put_bf16(A, row, f, kDesc, live ? X[(size_t)i * kDesc + f] : 0.f);
    put_bf16(A2, row, f, kDesc, live ? V[(size_t)i * kDesc + f] : 0.f);
  }
  if (warp == 0) tc_alloc(&s_taddr, 512);
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t T0 = s_taddr;
  const uint32_t tm = s_taddr + ((uint32_t)(32 * warp) << 16);
  uint32_t phase = 0;
  auto sync_issue = [&](auto&& issue) {
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      issue();
      tc_commit(&bar);
    }
    const bool got = mbar_wait(&bar, phase, status);
    phase ^= 1u;
    tc_fence_after();
    return __syncthreads_and(got);
  };
  // z1 = x W1^T and its tangent zd1 = v W1^T
  bool ok = sync_issue([&] {
    tc_gemm_issue(T0, A, sm + kFW1, kHid, kDesc, nullptr);
    tc_gemm_issue(T0 + 64, A2, sm + kFW1, kHid, kDesc, nullptr);
  });
  float h1[kHid], zd1[kHid];
  if (ok) {
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float z[16], zd[16];
      tc_ld16(tm + c0, z);
      tc_ld16(tm + 64 + c0, zd);
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int c = c0 + q;
        h1[c] = tanh_fast(z[q] + w.P[oB1 + c]);
        zd1[c] = zd[q];
        const float hd = (1.f - h1[c] * h1[c]) * zd[q];
        put_bf16(B, row, c, kHid, h1[c]);
        put_bf16(B2, row, c, kHid, hd);
        put_bf16(BT, c, row, 128, h1[c]);
        put_bf16(BT2, c, row, 128, hd);
      }
    }
    ok = sync_issue([&] {
      tc_gemm_issue(T0 + 128, B, sm + kFW2, kHid, kHid, nullptr);
      tc_gemm_issue(T0 + 192, B2, sm + kFW2, kHid, kHid, nullptr);
    });
  }
  if (ok) {
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float z[16], zd[16];
      tc_ld16(tm + 128 + c0, z);
      tc_ld16(tm + 192 + c0, zd);
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int c = c0 + q;
        const float h2 = tanh_fast(z[q] + w.P[oB2 + c]);
        const float s2 = 1.f - h2 * h2;
        const float w3 = w.P[oW3 + c];
        const float hd2 = s2 * zd[q];
        const float a_zd2 = live ? w3 * s2 : 0.f;
        const float a_z2 = w3 * (-2.f * h2 * zd[q]) * s2;
        const float gw3 = col_sum(hd2), gb2 = col_sum(a_z2);
        if (lane == 0) {
          atomicAdd(&grad[oW3 + c], gw3);
          atomicAdd(&grad[oB2 + c], gb2);
        }
        put_bf16(A, row, c, kHid, a_z2);
        put_bf16(A2, row, c, kHid, a_zd2);
        put_bf16(AT, c, row, 128, a_z2);
        put_bf16(AT2, c, row, 128, a_zd2);
      }
    }
    // W2 gradient a_z2^T h1 + a_zd2^T hd1; a_h1 = a_z2 W2; a_hd1 = a_zd2 W2
    ok = sync_issue([&] {
      tc_gemm_issue(T0 + 256, AT, BT, kHid, 128, nullptr);
      tc_gemm_issue(T0 + 256, AT2, BT2, kHid, 128, nullptr, true);
      tc_gemm_issue(T0, A, sm + kFW2T, kHid, kHid, nullptr);
      tc_gemm_issue(T0 + 64, A2, sm + kFW2T, kHid, kHid, nullptr);
    });
  }
  if (ok) {
    if (warp < 2) {
      for (int c0 = 0; c0 < kHid; c0 += 16) {
        float g[16];
        tc_ld16(tm + 256 + c0, g);
#pragma unroll
        for (int q = 0; q < 16; q++) atomicAdd(&grad[oW2 + row * kHid + c0 + q], g[q]);
      }
    }
    for (int c0 = 0; c0 < kHid; c0 += 16) {
      float ah[16], ahd[16];
      tc_ld16(tm + c0, ah);
      tc_ld16(tm + 64 + c0, ahd);
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int c = c0 + q;
        const float s1 = 1.f - h1[c] * h1[c];
        const float a_zd1 = ahd[q] * s1;
        const float a_z1 = (ah[q] + ahd[q] * (-2.f * h1[c] * zd1[c])) * s1;
        const float gb1 = col_sum(a_z1);
        if (lane == 0) atomicAdd(&grad[oB1 + c], gb1);
        put_bf16(AT, c, row, 128, a_z1);
        put_bf16(AT2, c, row, 128, a_zd1);
      }
    }
    for (int f = 0; f < kDesc; f++) {
      put_bf16(BT, f, row, 128, live ? X[(size_t)i * kDesc + f] : 0.f);
      put_bf16(BT2, f, row, 128, live ? V[(size_t)i * kDesc + f] : 0.f);
    }
    // W1 gradient a_z1^T x + a_zd1^T v
    ok = sync_issue([&] {
      tc_gemm_issue(T0 + 320, AT, BT, kDesc, 128, nullptr);
      tc_gemm_issue(T0 + 320, AT2, BT2, kDesc, 128, nullptr, true);
    });
  }
  if (ok && warp < 2) {
    for (int c0 = 0; c0 < kDesc; c0 += 16) {
      float g[16];
      tc_ld16(tm + 320 + c0, g);
#pragma unroll
      for (int q = 0; q < 16; q++) atomicAdd(&grad[oW1 + row * kDesc + c0 + q], g[q]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(s_taddr, 512);
}

// Adam (Kingma & Ba): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
// p -= lr mhat / (sqrt(vhat) + eps); then the BF16 operand copies
__global__ void k_adam(float* __restrict__ P, float* __restrict__ M, float* __restrict__ V,
                       const float* __restrict__ G, int step, float lr, float b1, float b2,
                       float eps) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kParams) return;
  const float g = G[k];
  const float m = b1 * M[k] + (1.f - b1) * g;
  const float v = b2 * V[k] + (1.f - b2) * g * g;
  M[k] = m;
  V[k] = v;
  const float mh = m / (1.f - powf(b1, (float)step));
  const float vh = v / (1.f - powf(b2, (float)step));
  P[k] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_net_cast(const float* __restrict__ P, __nv_bfloat16* W1, __nv_bfloat16* W1T,
                           __nv_bfloat16* W2, __nv_bfloat16* W2T) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < kHid * kDesc) {
    const int o = k / kDesc, in = k % kDesc;
    const __nv_bfloat16 b = __float2bfloat16_rn(P[oW1 + k]);
    W1[k] = b;
    W1T[in * kHid + o] = b;
  }
  if (k < kHid * kHid) {
    const int o = k / kHid, in = k % kHid;
    const __nv_bfloat16 b = __float2bfloat16_rn(P[oW2 + k]);
    W2[k] = b;
    W2T[in * kHid + o] = b;
  }
}

// energy E_i = mu + sigma t_i; gcoef = sigma * dt/dx * istd; block sums of E
__global__ void k_sg_scale(const float* __restrict__ t, const float* __restrict__ dtdx, int n,
                           double mu, double sigma, const float* __restrict__ istd,
                           float* __restrict__ gcoef, double* __restrict__ eatom) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (eatom) eatom[i] = mu + sigma * (double)t[i];
  for (int f = 0; f < kDesc; f++)
    gcoef[(size_t)i * kDesc + f] = (float)sigma * dtdx[(size_t)i * kDesc + f] * istd[f];
}

__global__ void k_sum_d(const double* __restrict__ v, int n, double* __restrict__ out) {
  __shared__ double sm[256];
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) s += v[k];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sm[0];
}

// sum |a - b|^2 and |b|^2 over 3n values (relative RMS of a against b),
// block partials added into out[0..1] (zeroed by the caller)
__global__ void k_err2(const double* __restrict__ a, const double* __restrict__ b, int n3,
                       double* __restrict__ out) {
  __shared__ double s1[256], s2[256];
  double x = 0.0, y = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n3; k += gridDim.x * blockDim.x) {
    const double d = a[k] - b[k];
    x += d * d;
    y += b[k] * b[k];
  }
  s1[threadIdx.x] = x;
  s2[threadIdx.x] = y;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&out[0], s1[0]);
    atomicAdd(&out[1], s2[0]);
  }
}

// ------------------------------------------------------------ host side

template <typename T>
cudaError_t sur_grow(T*& p, long long& have, long long need) {
  if (need <= have && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cudaError_t e = cudaMalloc(&p, sizeof(T) * (size_t)(need > 0 ? need : 1));
  have = e == cudaSuccess ? need : 0;
  return e;
}

NetDev net_of(const Surrogate& s) {
  NetDev w;
  w.W1 = s.W1;
  w.W1T = s.W1T;
  w.W2 = s.W2;
  w.W2T = s.W2T;
  w.P = s.P_d;
  return w;
}

__global__ void k_normalise(const float* __restrict__ G, const double* __restrict__ E, int n,
                            const float* __restrict__ mean, const float* __restrict__ istd,
                            double mu, double sigma, float* __restrict__ X,
                            float* __restrict__ T) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  for (int f = 0; f < kDesc; f++)
    X[(size_t)k * kDesc + f] = (G[(size_t)k * kDesc + f] - mean[f]) * istd[f];
  T[k] = (float)((E[k] - mu) / sigma);
}

__global__ void k_collect(const float* __restrict__ Graw, const double* __restrict__ eatom,
                          int n, int stride, int offset, float* __restrict__ SG,
                          double* __restrict__ SE, int base) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = offset + q * stride;
  if (i >= n) return;
  for (int f = 0; f < kDesc; f++) SG[(size_t)(base + q) * kDesc + f] = Graw[(size_t)i * kDesc + f];
  SE[base + q] = eatom[i];
}

inline int sblocks(long long n, int t) { return (int)((n + t - 1) / t); }

bool attrs_set = false;
// ---- the direct-force head: 32 -> H (tanh) -> H (tanh) -> 32, FP32 ----
// The second model kind.  Its 32 outputs w_i per atom, scaled to gcoef_i =
// w_i * s_out * istd (descriptor units; s_out = fh_out), take the place of the energy
// network's dE_i/dG_i in k_sg_force: F_j = -sum_i gcoef_i . dG_i/dr_j.
// Nothing makes gcoef a gradient, so the forces need not be conservative,
// as the reference's bond-order forces are not.  FP32 on the CUDA cores: the
// outputs multiply the descriptor derivatives directly, so BF16 weights would
// bound the force error near 1e-3; at 8-33 K parameters and one thread per
// atom the layers take tens of microseconds per 32,768 atoms.
// Parameters: W1 [H][32], b1 [H], W2 [H][H], b2 [H], W3 [32][H], b3 [32].
__host__ __device__ constexpr int fh_params(int H) { return H * 32 + H + H * H + H + 32 * H + 32; }

// forward, one thread per atom (weights in shared memory, read as broadcasts):
// gcoef (atom-major) and, for training, the input and hidden activations
// feature-major (xT[d n + i], h1T[j n + i], h2T[j n + i])
template <int H>
__global__ void __launch_bounds__(128)
    k_fh_forward(const float* __restrict__ X, int n, const float* __restrict__ P,
                 const float* __restrict__ gscale, float* __restrict__ gcoef,
                 float* __restrict__ xT, float* __restrict__ h1T, float* __restrict__ h2T) {
  extern __shared__ float wsm[];
  for (int k = threadIdx.x; k < fh_params(H); k += blockDim.x) wsm[k] = P[k];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *W1 = wsm, *b1 = W1 + H * 32, *W2 = b1 + H, *b2 = W2 + H * H, *W3 = b2 + H,
              *b3 = W3 + 32 * H;
  float x[32];
#pragma unroll
  for (int d = 0; d < 32; d++) {
    x[d] = X[(size_t)i * 32 + d];
    if (xT) xT[(size_t)d * n + i] = x[d];
  }
  float h1[H];
#pragma unroll
  for (int j = 0; j < H; j++) {
    float a = b1[j];
#pragma unroll
    for (int d = 0; d < 32; d++) a = fmaf(W1[j * 32 + d], x[d], a);
    h1[j] = tanhf(a);
    if (h1T) h1T[(size_t)j * n + i] = h1[j];
  }
  float w[32];
#pragma unroll
  for (int d = 0; d < 32; d++) w[d] = b3[d];
#pragma unroll 1
  for (int j = 0; j < H; j++) {
    float a = b2[j];
#pragma unroll
    for (int k = 0; k < H; k++) a = fmaf(W2[j * H + k], h1[k], a);
    const float h = tanhf(a);
    if (h2T) h2T[(size_t)j * n + i] = h;
#pragma unroll
    for (int d = 0; d < 32; d++) w[d] = fmaf(W3[d * H + j], h, w[d]);
  }
#pragma unroll
  for (int d = 0; d < 32; d++) gcoef[(size_t)i * 32 + d] = gscale ? w[d] * gscale[d] : w[d];
}

// backward of sum_i v_i . w_i (v = dL/dw, atom-major): the output and hidden
// deltas, feature-major (d3T[d n + i], d2T[j n + i], d1T[k n + i])
template <int H>
__global__ void __launch_bounds__(128)
    k_fh_backward(const float* __restrict__ V, int n, const float* __restrict__ P,
                  const float* __restrict__ h1T, const float* __restrict__ h2T,
                  float* __restrict__ d1T, float* __restrict__ d2T, float* __restrict__ d3T) {
  extern __shared__ float wsm[];
  for (int k = threadIdx.x; k < fh_params(H); k += blockDim.x) wsm[k] = P[k];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *W2 = wsm + H * 32 + H, *W3 = W2 + H * H + H;
  float d3[32];
#pragma unroll
  for (int d = 0; d < 32; d++) {
    d3[d] = V[(size_t)i * 32 + d];
    d3T[(size_t)d * n + i] = d3[d];
  }
  float d2[H];
#pragma unroll
  for (int j = 0; j < H; j++) {
    float a = 0.f;
#pragma unroll
    for (int d = 0; d < 32; d++) a = fmaf(W3[d * H + j], d3[d], a);
    const float h = h2T[(size_t)j * n + i];
    d2[j] = a * (1.f - h * h);
    d2T[(size_t)j * n + i] = d2[j];
  }
#pragma unroll 1
  for (int k = 0; k < H; k++) {
    float a = 0.f;
#pragma unroll
    for (int j = 0; j < H; j++) a = fmaf(W2[j * H + k], d2[j], a);
    const float h = h1T[(size_t)k * n + i];
    d1T[(size_t)k * n + i] = a * (1.f - h * h);
  }
}

// G[j][k] += sum_i A[j][i] B[k][i] (A: J x n, B: K x n, feature-major) and,
// when gb is given, gb[j] += sum_i A[j][i]: 32 x 32 output tiles per block
// over a chunk of atoms, staged 64 atoms at a time, one atomic per output
constexpr int kOutChunk = 1024;
__global__ void __launch_bounds__(256)
    k_fh_outer(const float* __restrict__ A, const float* __restrict__ B, int n, int J, int K,
               float* __restrict__ G, float* __restrict__ gb) {
  __shared__ float as[32][65], bs[32][65];
  const int j0 = blockIdx.x * 32, k0 = blockIdx.y * 32, i0 = blockIdx.z * kOutChunk;
  const int tid = threadIdx.x, tj = tid >> 3, tk = (tid & 7) * 4;  // 32 x (8 x 4)
  float acc[4] = {0.f, 0.f, 0.f, 0.f}, bsum = 0.f;
  const int i1 = min(n, i0 + kOutChunk);
  for (int ib = i0; ib < i1; ib += 64) {
    for (int e = tid; e < 32 * 64; e += 256) {
      const int r = e >> 6, c = e & 63, ii = ib + c;
      as[r][c] = (j0 + r < J && ii < i1) ? A[(size_t)(j0 + r) * n + ii] : 0.f;
      bs[r][c] = (k0 + r < K && ii < i1) ? B[(size_t)(k0 + r) * n + ii] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < 64; c++) {
      const float a = as[tj][c];
      acc[0] = fmaf(a, bs[tk][c], acc[0]);
      acc[1] = fmaf(a, bs[tk + 1][c], acc[1]);
      acc[2] = fmaf(a, bs[tk + 2][c], acc[2]);
      acc[3] = fmaf(a, bs[tk + 3][c], acc[3]);
      if (gb && blockIdx.y == 0 && tk == 0) bsum += a;
    }
    __syncthreads();
  }
  if (j0 + tj < J) {
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (k0 + tk + u < K) atomicAdd(&G[(size_t)(j0 + tj) * K + k0 + tk + u], acc[u]);
    if (gb && blockIdx.y == 0 && tk == 0) atomicAdd(&gb[j0 + tj], bsum);
  }
}

// Adam over `count` parameters (the force head's; k_adam's rule)
__global__ void k_adam_n(float* __restrict__ P, float* __restrict__ M, float* __restrict__ V,
                         const float* __restrict__ G, int count, int step, float lr, float b1,
                         float b2, float eps) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const float g = G[k];
  const float m = b1 * M[k] + (1.f - b1) * g;
  const float v = b2 * V[k] + (1.f - b2) * g * g;
  M[k] = m;
  V[k] = v;
  const float mh = m / (1.f - powf(b1, (float)step));
  const float vh = v / (1.f - powf(b2, (float)step));
  P[k] -= lr * mh / (sqrtf(vh) + eps);
}

// gscale_d = F_rms istd_d: the head's outputs in units of the force scale
__global__ void k_fh_gscale(const float* __restrict__ istd, float frms, float* __restrict__ gs) {
  if (threadIdx.x < 32) gs[threadIdx.x] = frms * istd[threadIdx.x];
}

__global__ void k_fill_nan(double* p) { *p = __longlong_as_double(0x7FF8000000000000LL); }

// floats as ints with the same order (negative values: the 31 low bits flipped)
__device__ __forceinline__ int ord_key(float f) {
  const int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7FFFFFFF;
}

// per-feature minimum and maximum of X (n32 = 32 n values, atom-major) as
// ordered keys; the grid's stride is a multiple of 32, so a thread keeps
// one feature
__global__ void k_feat_range(const float* __restrict__ X, long long n32, int* __restrict__ lo,
                             int* __restrict__ hi) {
  const int f = threadIdx.x & 31;
  int kl = INT_MAX, kh = INT_MIN;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n32;
       e += (long long)gridDim.x * blockDim.x) {
    const int k = ord_key(X[e]);
    kl = min(kl, k);
    kh = max(kh, k);
  }
  atomicMin(&lo[f], kl);
  atomicMax(&hi[f], kh);
}

// flag = 1 when a value of X lies outside [lo_f, hi_f] of its feature (or is NaN)
__global__ void k_range_check(const float* __restrict__ X, long long n32,
                              const float* __restrict__ lo, const float* __restrict__ hi,
                              int* __restrict__ flag) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool out = false;
  if (e < n32) {
    const float x = X[e];
    const int f = (int)(e & 31);
    out = !(x >= lo[f] && x <= hi[f]);
  }
  if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// probe outputs: w uniform on [-sqrt 3, sqrt 3] (unit variance, from a
// splitmix64 hash of the index), written as coefficients w istd_d
__global__ void k_fh_probe(float* __restrict__ gcoef, long long n32, const float* __restrict__ istd,
                           unsigned long long seed) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n32) return;
  unsigned long long z = seed + 0x9E3779B97F4A7C15ULL * (unsigned long long)(k + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  const float u = (float)(z >> 40) * (1.f / 16777216.f);  // [0, 1)
  gcoef[k] = (2.f * u - 1.f) * 1.7320508f * istd[k & 31];
}

// acc[0] += sum_k F[k]^2
__global__ void k_sumsq(const float* __restrict__ F, int n3, double* __restrict__ acc) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double s = k < n3 ? (double)F[k] * F[k] : 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(acc, s);
}

void set_attrs() {
  if (attrs_set) return;
  cudaFuncSetAttribute(k_net_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmInfer);
  cudaFuncSetAttribute(k_net_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmTrain);
  cudaFuncSetAttribute(k_net_train_force, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmForce);
  cudaFuncSetAttribute(k_fh_forward<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(float) * fh_params(128));
  cudaFuncSetAttribute(k_fh_backward<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(float) * fh_params(128));
  attrs_set = true;
}

double fh_out_scale(const Surrogate& s) {
  if (s.fh_out > 0.0) return s.fh_out;
  return sqrt(s.force_var > 0 ? s.force_var : 1.0);
}

// the direct-force head's launches for its width
void fh_forward(const Surrogate& s, const float* X, int n, float* gcoef, bool keep,
                cudaStream_t st) {
  const int B = (n + 127) / 128;
  const size_t sm = sizeof(float) * fh_params(s.fh_hidden);
  float* xT = keep ? s.fh_xT : nullptr;
  float* h1 = keep ? s.fh_h1T : nullptr;
  float* h2 = keep ? s.fh_h2T : nullptr;
  const float* gs = s.fh_gs;
  if (s.fh_hidden == 32)
    k_fh_forward<32><<<B, 128, sm, st>>>(X, n, s.FP_d, gs, gcoef, xT, h1, h2);
  else if (s.fh_hidden == 64)
    k_fh_forward<64><<<B, 128, sm, st>>>(X, n, s.FP_d, gs, gcoef, xT, h1, h2);
  else
    k_fh_forward<128><<<B, 128, sm, st>>>(X, n, s.FP_d, gs, gcoef, xT, h1, h2);
}

// FG += d(sum_i v_i . w_i)/dparams for the activations of the last kept forward
void fh_backward(Surrogate& s, const float* V, int n, cudaStream_t st) {
  const int H = s.fh_hidden, B = (n + 127) / 128;
  const size_t sm = sizeof(float) * fh_params(H);
  if (H == 32)
    k_fh_backward<32><<<B, 128, sm, st>>>(V, n, s.FP_d, s.fh_h1T, s.fh_h2T, s.fh_d1T, s.fh_d2T,
                                          s.fh_d3T);
  else if (H == 64)
    k_fh_backward<64><<<B, 128, sm, st>>>(V, n, s.FP_d, s.fh_h1T, s.fh_h2T, s.fh_d1T, s.fh_d2T,
                                          s.fh_d3T);
  else
    k_fh_backward<128><<<B, 128, sm, st>>>(V, n, s.FP_d, s.fh_h1T, s.fh_h2T, s.fh_d1T,
                                           s.fh_d2T, s.fh_d3T);
  float* G = s.FG_d;
  float *gW1 = G, *gb1 = gW1 + H * 32, *gW2 = gb1 + H, *gb2 = gW2 + H * H, *gW3 = gb2 + H,
        *gb3 = gW3 + 32 * H;
  const int nz = (n + kOutChunk - 1) / kOutChunk;
  const int hb = (H + 31) / 32;
  k_fh_outer<<<dim3(1, hb, nz), 256, 0, st>>>(s.fh_d3T, s.fh_h2T, n, 32, H, gW3, gb3);
  k_fh_outer<<<dim3(hb, hb, nz), 256, 0, st>>>(s.fh_d2T, s.fh_h1T, n, H, H, gW2, gb2);
  k_fh_outer<<<dim3(hb, 1, nz), 256, 0, st>>>(s.fh_d1T, s.fh_xT, n, H, 32, gW1, gb1);
}

cudaError_t fh_scratch(Surrogate& s, long long n) {
  if (n <= s.fh_n) return cudaSuccess;
  cudaError_t e;
  const long long H = s.fh_hidden;
  for (float** p : {&s.fh_h1T, &s.fh_h2T, &s.fh_d1T, &s.fh_d2T}) {
    long long h = 0;
    if (*p) cudaFree(*p);
    *p = nullptr;
    if ((e = sur_grow(*p, h, H * n)) != cudaSuccess) return e;
  }
  for (float** p : {&s.fh_xT, &s.fh_d3T}) {
    long long h = 0;
    if (*p) cudaFree(*p);
    *p = nullptr;
    if ((e = sur_grow(*p, h, 32 * n)) != cudaSuccess) return e;
  }
  s.fh_n = n;
  return cudaSuccess;
}

}  // namespace

int sur_fh_param_count(int hidden) { return fh_params(hidden); }

int sur_set_model(Surrogate& s, int kind, int hidden, cudaStream_t st) {
  if (kind == 0) {
    s.kind = 0;
    return 0;
  }
  if (kind != 1 || !(hidden == 32 || hidden == 64 || hidden == 128)) return -1;
  set_attrs();
  s.kind = 1;
  if (hidden != s.fh_hidden) s.fh_n = 0;  // activations are per width
  s.fh_hidden = hidden;
  s.fh_np = fh_params(hidden);
  cudaError_t e;
  for (float** p : {&s.FP_d, &s.FM_d, &s.FV_d, &s.FG_d}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    long long h = 0;
    if ((e = sur_grow(*p, h, s.fh_np)) != cudaSuccess) return e;
  }
  if (!s.fh_gs) {
    long long h = 0;
    if ((e = sur_grow(s.fh_gs, h, 32)) != cudaSuccess) return e;
  }
  // weights from the surrogate's seed (another stream of the LCG than the
  // energy network's), zero biases
  const int H = hidden;
  std::vector<float> P(s.fh_np, 0.f);
  unsigned long long x = (s.seed ^ 0x9E3779B97F4A7C15ULL) * 6364136223846793005ULL + 1;
  auto uni = [&]() {
    x = x * 6364136223846793005ULL + 1442695040888963407ULL;
    return (float)((x >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
  };
  // hidden layers Xavier-uniform; output layer zero, so that training starts
  // from zero forces (loss 1) rather than from forces many times F_rms
  const float a1 = sqrtf(6.f / (32 + H)), a2 = sqrtf(6.f / (H + H));
  for (int k = 0; k < H * 32; k++) P[k] = a1 * uni();
  for (int k = 0; k < H * H; k++) P[H * 32 + H + k] = a2 * uni();
  return sur_fh_params(s, P.data(), s.fh_np, true, st);
}

int sur_fh_params(Surrogate& s, float* P, int count, bool set, cudaStream_t st) {
  if (s.kind != 1 || count != s.fh_np) return -1;
  cudaError_t e;
  if (set) {
    if ((e = cudaMemcpyAsync(s.FP_d, P, sizeof(float) * count, cudaMemcpyHostToDevice, st)) !=
        cudaSuccess)
      return e;
    cudaMemsetAsync(s.FM_d, 0, sizeof(float) * count, st);
    cudaMemsetAsync(s.FV_d, 0, sizeof(float) * count, st);
    s.fh_step = 0;
  } else if ((e = cudaMemcpyAsync(P, s.FP_d, sizeof(float) * count, cudaMemcpyDeviceToHost,
                                  st)) != cudaSuccess) {
    return e;
  }
  return cudaStreamSynchronize(st);
}

int sur_fh_grad(Surrogate& s, const float* X, const float* V, int n, float* grad,
                cudaStream_t st) {
  if (s.kind != 1) return -1;
  cudaError_t e;
  float *dX = nullptr, *dV = nullptr, *dw = nullptr;
  if ((e = fh_scratch(s, n)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&dX, sizeof(float) * 32 * n)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&dV, sizeof(float) * 32 * n)) != cudaSuccess ||
      (e = cudaMalloc(&dw, sizeof(float) * 32 * n)) != cudaSuccess) {
    cudaFree(dX);
    if (dV) cudaFree(dV);
    return e;
  }
  cudaMemcpyAsync(dX, X, sizeof(float) * 32 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dV, V, sizeof(float) * 32 * n, cudaMemcpyHostToDevice, st);
  // raw outputs (no scaling) with the activations kept
  const float* gs = s.fh_gs;
  s.fh_gs = nullptr;
  fh_forward(s, dX, n, dw, true, st);
  s.fh_gs = const_cast<float*>(gs);
  cudaMemsetAsync(s.FG_d, 0, sizeof(float) * s.fh_np, st);
  fh_backward(s, dV, n, st);
  cudaMemcpyAsync(grad, s.FG_d, sizeof(float) * s.fh_np, cudaMemcpyDeviceToHost, st);
  e = cudaStreamSynchronize(st);
  cudaFree(dX);
  cudaFree(dV);
  cudaFree(dw);
  if (e != cudaSuccess) return e;
  return (int)cudaGetLastError();
}

int sur_init(Surrogate& s, unsigned long long seed, cudaStream_t st) {
  cudaError_t e;
  s.P = default_desc(s.rc);
  long long h = 0;
  for (float** p : {&s.P_d, &s.M_d, &s.V_d, &s.G_d}) {
    h = 0;
    if ((e = sur_grow(*p, h, kParams)) != cudaSuccess) return e;
  }
  for (__nv_bfloat16** p : {&s.W1, &s.W1T, &s.W2, &s.W2T}) {
    h = 0;
    if ((e = sur_grow(*p, h, kHid * kHid)) != cudaSuccess) return e;
  }
  for (float** p : {&s.mean_d, &s.istd_d}) {
    h = 0;
    if ((e = sur_grow(*p, h, kDesc)) != cudaSuccess) return e;
  }
  h = 0;
  if ((e = sur_grow(s.loss_d, h, 4)) != cudaSuccess) return e;
  h = 0;
  if ((e = sur_grow(s.scratch, h, 8)) != cudaSuccess) return e;
  h = 0;
  if ((e = sur_grow(s.status_d, h, 1)) != cudaSuccess) return e;
  cudaMemsetAsync(s.status_d, 0, sizeof(int), st);
  s.seed = seed;
  // Xavier-uniform weights from a 64-bit LCG, zero biases
  std::vector<float> P(kParams, 0.f);
  unsigned long long x = seed * 6364136223846793005ULL + 1442695040888963407ULL;
  auto uni = [&]() {
    x = x * 6364136223846793005ULL + 1442695040888963407ULL;
    return (float)((x >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
  };
  const float a1 = sqrtf(6.f / (kDesc + kHid)), a2 = sqrtf(6.f / (kHid + kHid)),
              a3 = sqrtf(6.f / (kHid + 1));
  for (int k = 0; k < kHid * kDesc; k++) P[oW1 + k] = a1 * uni();
  for (int k = 0; k < kHid * kHid; k++) P[oW2 + k] = a2 * uni();
  for (int k = 0; k < kHid; k++) P[oW3 + k] = a3 * uni();
  return sur_set_params(s, P.data(), st);
}

int sur_set_params(Surrogate& s, const float* P, cudaStream_t st) {
  cudaError_t e;
  if ((e = cudaMemcpyAsync(s.P_d, P, sizeof(float) * kParams, cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return e;
  cudaMemsetAsync(s.M_d, 0, sizeof(float) * kParams, st);
  cudaMemsetAsync(s.V_d, 0, sizeof(float) * kParams, st);
  s.adam_step = 0;
  k_net_cast<<<sblocks(kHid * kHid, 256), 256, 0, st>>>(s.P_d, s.W1, s.W1T, s.W2, s.W2T);
  return cudaStreamSynchronize(st);
}

int sur_get_params(const Surrogate& s, float* P, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(P, s.P_d, sizeof(float) * kParams, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

int sur_param_count() { return kParams; }

// neighbours, then descriptors (normalised when `normalised`) for atoms [0, n)
// q_if = sum_j (e_j - e_i) . dG_if/dd_j for host e3 (n x 3) on the short
// lists of the last sur_descriptors call; q_host n x 32
int sur_directional(Surrogate& s, const md_double4* pos, int n, double box, const double* e3,
                    double* q_host, cudaStream_t st) {
  if (n <= 0) return 0;
  std::vector<float> he(3 * (size_t)n);
  for (size_t k = 0; k < he.size(); k++) he[k] = (float)e3[k];
  float *de = nullptr, *dv = nullptr;
  cudaError_t e = cudaMalloc(&de, sizeof(float) * he.size());
  if (e == cudaSuccess) e = cudaMalloc(&dv, sizeof(float) * kDesc * (size_t)n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(de, he.data(), sizeof(float) * he.size(), cudaMemcpyHostToDevice, st);
  std::vector<float> hv(kDesc * (size_t)n);
  if (e == cudaSuccess) {
    k_sg_ctrans<<<sblocks(n, 4), 128, 0, st>>>(pos, n, s.sl, s.slen, box, s.P, de, 1.f, nullptr,
                                               dv);
    e = cudaMemcpyAsync(hv.data(), dv, sizeof(float) * hv.size(), cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess)
    for (size_t k = 0; k < hv.size(); k++) q_host[k] = hv[k];
  if (de) cudaFree(de);
  if (dv) cudaFree(dv);
  return (int)e;
}

int sur_descriptors(Surrogate& s, const md_double4* pos, int n, const RowWalker& w,
                    bool normalised, int* d_status, cudaStream_t st) {
  cudaError_t e;
  if ((e = sur_grow(s.sl, s.n_sl, (long long)n * kSgMax)) != cudaSuccess) return e;
  long long h = s.n_alloc;
  if (n > s.n_alloc) {
    for (float** p : {&s.X, &s.dtdx, &s.gcoef}) {
      h = 0;
      if ((e = sur_grow(*p, h, (long long)n * kDesc)) != cudaSuccess) return e;
    }
    h = 0;
    if ((e = sur_grow(s.t, h, n)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.F32, h, 3LL * n)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.eatom, h, n)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.slen, h, n)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.pos32, h, n)) != cudaSuccess) return e;
    s.n_alloc = n;
  }
  if (n == 0) return 0;
  k_sg_pos32<<<sblocks(n, 256), 256, 0, st>>>(pos, n, s.pos32);
  k_sg_short<<<sblocks(n, 4), 128, 0, st>>>(s.pos32, w, s.rc, s.sl, s.slen, d_status);
  k_sg_desc<<<sblocks(n, 4), 128, 0, st>>>(pos, n, s.sl, s.slen, w.g.box, s.P,
                                             normalised ? s.mean_d : nullptr,
                                             normalised ? s.istd_d : nullptr, s.X);
  return (int)cudaGetLastError();
}

int sur_collect(Surrogate& s, int n, const double* eatom, int stride, int offset,
                cudaStream_t st, int* added) {
  cudaError_t e;
  const int cnt = offset < n ? (n - offset + stride - 1) / stride : 0;
  if (s.ns + cnt > s.ns_cap) {
    const long long cap = std::max<long long>(2LL * (s.ns + cnt), 4096);
    float* nG = nullptr;
    double* nE = nullptr;
    if ((e = cudaMalloc(&nG, sizeof(float) * kDesc * cap)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&nE, sizeof(double) * cap)) != cudaSuccess) {
      cudaFree(nG);
      return e;
    }
    if (s.ns > 0) {
      cudaMemcpyAsync(nG, s.SG, sizeof(float) * kDesc * s.ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(nE, s.SE, sizeof(double) * s.ns, cudaMemcpyDeviceToDevice, st);
    }
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    if (s.SG) cudaFree(s.SG);
    if (s.SE) cudaFree(s.SE);
    s.SG = nG;
    s.SE = nE;
    s.ns_cap = (int)cap;
  }
  if (cnt > 0)
    k_collect<<<sblocks(cnt, 256), 256, 0, st>>>(s.X, eatom, n, stride, offset, s.SG, s.SE, s.ns);
  s.ns += cnt;
  if (added) *added = cnt;
  return (int)cudaGetLastError();
}

// fixes the input/target normalisation from the samples (first training)
namespace {
int sur_normalise(Surrogate& s, cudaStream_t st) {
  std::vector<float> G((size_t)s.ns * kDesc);
  std::vector<double> E(s.ns);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(G.data(), s.SG, sizeof(float) * G.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(E.data(), s.SE, sizeof(double) * E.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return e;
  float mean[kDesc], istd[kDesc];
  for (int f = 0; f < kDesc; f++) {
    double m = 0, v = 0;
    for (int k = 0; k < s.ns; k++) m += G[(size_t)k * kDesc + f];
    m /= s.ns;
    for (int k = 0; k < s.ns; k++) {
      const double d = G[(size_t)k * kDesc + f] - m;
      v += d * d;
    }
    v /= s.ns;
    mean[f] = (float)m;
    istd[f] = (float)(1.0 / sqrt(v + 1e-12));
  }
  double mu = 0, var = 0;
  for (double x : E) mu += x;
  mu /= s.ns;
  for (double x : E) var += (x - mu) * (x - mu);
  var /= s.ns;
  s.mu = mu;
  s.sigma = sqrt(var) > 0 ? sqrt(var) : 1.0;
  cudaMemcpyAsync(s.mean_d, mean, sizeof(mean), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s.istd_d, istd, sizeof(istd), cudaMemcpyHostToDevice, st);
  s.normalised = true;
  s.fh_out = 0.0;  // measured again for the new normalisation
  return cudaStreamSynchronize(st);
}
}  // namespace

int sur_train(Surrogate& s, int steps, int batch, float lr, double* loss_out, cudaStream_t st) {
  if (s.ns < 1) return -1;
  cudaError_t e;
  set_attrs();
  if (!s.normalised) {
    int r = sur_normalise(s, st);
    if (r) return r;
  }
  long long h = s.nsx;
  if ((e = sur_grow(s.SX, h, (long long)s.ns * kDesc)) != cudaSuccess) return e;
  h = s.nsx;
  if ((e = sur_grow(s.ST, h, s.ns)) != cudaSuccess) return e;
  s.nsx = s.ns;
  k_normalise<<<sblocks(s.ns, 256), 256, 0, st>>>(s.SG, s.SE, s.ns, s.mean_d, s.istd_d, s.mu,
                                                  s.sigma, s.SX, s.ST);
  const int tiles = (batch + 127) / 128;
  const float inv = 1.f / (float)(tiles * 128);
  double acc = 0;
  int nacc = 0;
  for (int it = 0; it < steps; it++) {
    cudaMemsetAsync(s.G_d, 0, sizeof(float) * kParams, st);
    cudaMemsetAsync(s.loss_d, 0, sizeof(double), st);
    k_net_train<<<tiles, 128, kSmTrain, st>>>(s.SX, s.ST, s.ns, nullptr, tiles * 128,
                                              s.seed + 0x9E37ULL * (unsigned long long)(s.adam_step + 1),
                                              net_of(s), inv, s.G_d, s.loss_d, s.status_d);
    s.adam_step++;
    k_adam<<<sblocks(kParams, 256), 256, 0, st>>>(s.P_d, s.M_d, s.V_d, s.G_d, s.adam_step, lr,
                                                 0.9f, 0.999f, 1e-8f);
    k_net_cast<<<sblocks(kHid * kHid, 256), 256, 0, st>>>(s.P_d, s.W1, s.W1T, s.W2, s.W2T);
    if (it >= steps - 16) {  // mean loss of the last steps
      double l = 0;
      cudaMemcpyAsync(&l, s.loss_d, sizeof(double), cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
      acc += l;
      nacc++;
    }
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  if (loss_out) *loss_out = nacc ? acc / nacc : 0.0;
  return (int)cudaGetLastError();
}

int sur_loss_grad(Surrogate& s, const float* X, const float* T, int n, float* grad,
                  double* loss, cudaStream_t st) {
  cudaError_t e;
  set_attrs();
  long long h = s.nxg;
  if ((e = sur_grow(s.Xg, h, (long long)n * kDesc)) != cudaSuccess) return e;
  h = s.nxg;
  if ((e = sur_grow(s.Tg, h, n)) != cudaSuccess) return e;
  h = s.nxg;
  if ((e = sur_grow(s.rows_d, h, n)) != cudaSuccess) return e;
  s.nxg = n;
  std::vector<int> rows(n);
  for (int k = 0; k < n; k++) rows[k] = k;
  cudaMemcpyAsync(s.Xg, X, sizeof(float) * kDesc * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s.Tg, T, sizeof(float) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s.rows_d, rows.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(s.G_d, 0, sizeof(float) * kParams, st);
  cudaMemsetAsync(s.loss_d, 0, sizeof(double), st);
  k_net_train<<<(n + 127) / 128, 128, kSmTrain, st>>>(s.Xg, s.Tg, n, s.rows_d, n, 0ULL,
                                                      net_of(s), 1.f / (float)n, s.G_d,
                                                      s.loss_d, s.status_d);
  cudaMemcpyAsync(grad, s.G_d, sizeof(float) * kParams, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(loss, s.loss_d, sizeof(double), cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  return (int)cudaGetLastError();
}

// network outputs for given normalised inputs: t (n) and dt/dx (n x 32)
int sur_net_eval(Surrogate& s, const float* X, int n, float* t, float* dtdx, cudaStream_t st) {
  cudaError_t e;
  set_attrs();
  long long h = s.nxg;
  if ((e = sur_grow(s.Xg, h, (long long)n * kDesc)) != cudaSuccess) return e;
  h = s.nxg;
  if ((e = sur_grow(s.Tg, h, (long long)n * (kDesc + 1))) != cudaSuccess) return e;
  s.nxg = n;
  cudaMemcpyAsync(s.Xg, X, sizeof(float) * kDesc * n, cudaMemcpyHostToDevice, st);
  k_net_infer<<<(n + 127) / 128, 128, kSmInfer, st>>>(s.Xg, n, net_of(s), s.Tg, s.Tg + n,
                                                     s.status_d);
  cudaMemcpyAsync(t, s.Tg, sizeof(float) * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(dtdx, s.Tg + n, sizeof(float) * kDesc * n, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  return (int)cudaGetLastError();
}

// bond-order forces (into f3, added when accumulate) and per-atom energies
// of atoms [0, n) from the network; energy_dev (optional) gets their sum
int sur_forces(Surrogate& s, const md_double4* pos, int n, const RowWalker& w, double* f3,
               int accumulate, double* energy_dev, int* d_status, cudaStream_t st,
               bool* declined, int* run_exact, int* declined_count) {
  if (!s.normalised) return -1;
  set_attrs();
  int r = sur_descriptors(s, pos, n, w, true, d_status, st);
  if (r) return r;
  if (n == 0) return 0;
  const int* skip = nullptr;
  if (run_exact) {
    // the decision stays on the device: the store below and the caller's
    // exact kernels read the flag
    cudaMemsetAsync(run_exact, 0, sizeof(int), st);
    if (s.have_range) {
      k_range_check<<<sblocks(32LL * n, 256), 256, 0, st>>>(s.X, 32LL * n, s.xlo_d, s.xhi_d,
                                                            run_exact);
      skip = run_exact;
    }
  } else if (declined) {
    *declined = false;
    if (s.have_range) {
      // outside the training data's descriptor range the model is not used
      cudaMemsetAsync(s.oor_d, 0, sizeof(int), st);
      k_range_check<<<sblocks(32LL * n, 256), 256, 0, st>>>(s.X, 32LL * n, s.xlo_d, s.xhi_d,
                                                            s.oor_d);
      int flag = 0;
      cudaError_t e = cudaMemcpyAsync(&flag, s.oor_d, sizeof(int), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return e;
      if (flag) {
        *declined = true;
        return 0;
      }
    }
  }
  if (s.kind == 1) {
    // the direct-force head: coefficients straight from the network; it
    // models forces only, so the energy it reports is NaN
    k_fh_gscale<<<1, 32, 0, st>>>(s.istd_d, (float)fh_out_scale(s), s.fh_gs);
    fh_forward(s, s.X, n, s.gcoef, false, st);
    cudaMemsetAsync(s.F32, 0, sizeof(float) * 3 * (size_t)n, st);
    k_sg_force<<<sblocks(n, 4), 128, 0, st>>>(pos, n, s.sl, s.slen, w.g.box, s.P, s.gcoef, s.F32);
    k_sg_store<<<sblocks(3LL * n, 256), 256, 0, st>>>(s.F32, f3, n, accumulate, skip,
                                                      declined_count);
    if (energy_dev) k_fill_nan<<<1, 1, 0, st>>>(energy_dev);
    return (int)cudaGetLastError();
  }
  k_net_infer<<<(n + 127) / 128, 128, kSmInfer, st>>>(s.X, n, net_of(s), s.t, s.dtdx, s.status_d);
  k_sg_scale<<<sblocks(n, 256), 256, 0, st>>>(s.t, s.dtdx, n, s.mu, s.sigma, s.istd_d, s.gcoef,
                                              s.eatom);
  cudaMemsetAsync(s.F32, 0, sizeof(float) * 3 * (size_t)n, st);
  k_sg_force<<<sblocks(n, 4), 128, 0, st>>>(pos, n, s.sl, s.slen, w.g.box, s.P, s.gcoef, s.F32);
  k_sg_store<<<sblocks(3LL * n, 256), 256, 0, st>>>(s.F32, f3, n, accumulate, skip,
                                                    declined_count);
  if (energy_dev) k_sum_d<<<1, 256, 0, st>>>(s.eatom, n, energy_dev);
  return (int)cudaGetLastError();
}

int sur_add_config(Surrogate& s, const md_double4* pos, int n, double box, const double* fx,
                   const double* eatom, cudaStream_t st) {
  SurConfig c;
  c.n = n;
  c.box = box;
  cudaError_t e;
  if ((e = cudaMalloc(&c.pos, sizeof(md_double4) * n)) != cudaSuccess ||
      (e = cudaMalloc(&c.sl, sizeof(uint32_t) * (size_t)n * kSgMax)) != cudaSuccess ||
      (e = cudaMalloc(&c.slen, sizeof(int) * n)) != cudaSuccess ||
      (e = cudaMalloc(&c.fx, sizeof(double) * 3 * n)) != cudaSuccess ||
      (e = cudaMalloc(&c.eatom, sizeof(double) * n)) != cudaSuccess ||
      (e = cudaMalloc(&c.G, sizeof(float) * kDesc * n)) != cudaSuccess) {
    for (void* p : {(void*)c.pos, (void*)c.sl, (void*)c.slen, (void*)c.fx, (void*)c.eatom,
                    (void*)c.G})
      if (p) cudaFree(p);
    return e;
  }
  cudaMemcpyAsync(c.pos, pos, sizeof(md_double4) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c.sl, s.sl, sizeof(uint32_t) * (size_t)n * kSgMax, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c.slen, s.slen, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c.fx, fx, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c.eatom, eatom, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c.G, s.X, sizeof(float) * kDesc * n, cudaMemcpyDeviceToDevice, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  s.cfgs.push_back(c);
  return 0;
}

namespace {
// normalisation from the stored configurations (first training)
int sur_normalise_cfgs(Surrogate& s, cudaStream_t st) {
  double sum[kDesc] = {0}, sq[kDesc] = {0}, esum = 0, esq = 0, fsq = 0;
  long long cnt = 0;
  for (const SurConfig& c : s.cfgs) {
    std::vector<float> G((size_t)c.n * kDesc);
    std::vector<double> E(c.n), F(3 * (size_t)c.n);
    cudaMemcpyAsync(G.data(), c.G, sizeof(float) * G.size(), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(E.data(), c.eatom, sizeof(double) * E.size(), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(F.data(), c.fx, sizeof(double) * F.size(), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    for (int k = 0; k < c.n; k++) {
      for (int f = 0; f < kDesc; f++) {
        const double g = G[(size_t)k * kDesc + f];
        sum[f] += g;
        sq[f] += g * g;
      }
      esum += E[k];
      esq += E[k] * E[k];
    }
    for (double f : F) fsq += f * f;
    cnt += c.n;
  }
  float mean[kDesc], istd[kDesc];
  for (int f = 0; f < kDesc; f++) {
    const double m = sum[f] / cnt, v = sq[f] / cnt - m * m;
    mean[f] = (float)m;
    istd[f] = (float)(1.0 / sqrt(fmax(v, 0.0) + 1e-12));
  }
  s.mu = esum / cnt;
  const double ev = esq / cnt - s.mu * s.mu;
  s.sigma = ev > 0 ? sqrt(ev) : 1.0;
  s.force_var = fsq / (3.0 * cnt) > 0 ? fsq / (3.0 * cnt) : 1.0;
  cudaMemcpyAsync(s.mean_d, mean, sizeof(mean), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s.istd_d, istd, sizeof(istd), cudaMemcpyHostToDevice, st);
  s.normalised = true;
  s.fh_out = 0.0;  // measured again for the new normalisation
  return cudaStreamSynchronize(st);
}
}  // namespace

namespace {
// Force matching of the direct-force head: per Adam step one stored
// configuration, loss w_force mean(|F - F*|^2) / var_F, with
//   dL/dw_i = -2 kappa s_out istd . sum_j (F_j - F*_j) . dG_i/dr_j
// (s_out = fh_out, the force scale of one unit of output)
// from the same transpose as the energy network's force term (k_sg_ctrans),
// then the head's backward pass and Adam.
int train_fh(Surrogate& s, int steps, float lr, int nmax, double* loss_e, double* loss_f,
             cudaStream_t st) {
  cudaError_t e;
  if ((e = fh_scratch(s, nmax)) != cudaSuccess) return e;
  const int ncfg = (int)s.cfgs.size();
  if (s.fh_out <= 0.0) {
    // the output scale: force RMS per component from unit-variance outputs
    // on the first configuration
    const SurConfig& c = s.cfgs[0];
    k_fh_probe<<<sblocks(32LL * c.n, 256), 256, 0, st>>>(s.gcoef, 32LL * c.n, s.istd_d,
                                                         s.seed);
    cudaMemsetAsync(s.F32, 0, sizeof(float) * 3 * (size_t)c.n, st);
    k_sg_force<<<sblocks(c.n, 4), 128, 0, st>>>(c.pos, c.n, c.sl, c.slen, c.box, s.P, s.gcoef,
                                                s.F32);
    cudaMemsetAsync(s.scratch, 0, sizeof(double), st);
    k_sumsq<<<sblocks(3LL * c.n, 256), 256, 0, st>>>(s.F32, 3 * c.n, s.scratch);
    double sq = 0;
    cudaMemcpyAsync(&sq, s.scratch, sizeof(double), cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    const double rms = sqrt(sq / (3.0 * c.n));
    s.fh_out = rms > 0 ? sqrt(s.force_var) / rms : sqrt(s.force_var);
  }
  const float gsc = (float)s.fh_out;
  k_fh_gscale<<<1, 32, 0, st>>>(s.istd_d, gsc, s.fh_gs);
  double acc_f = 0;
  int nacc = 0;
  for (int it = 0; it < steps; it++) {
    const SurConfig& c = s.cfgs[(it * 7919 + (int)(s.seed % 101)) % ncfg];
    const int n = c.n;
    fh_forward(s, c.X, n, s.gcoef, true, st);
    cudaMemsetAsync(s.F32, 0, sizeof(float) * 3 * (size_t)n, st);
    k_sg_force<<<sblocks(n, 4), 128, 0, st>>>(c.pos, n, c.sl, c.slen, c.box, s.P, s.gcoef,
                                                s.F32);
    cudaMemsetAsync(s.scratch, 0, sizeof(double) * 2, st);
    k_fm_resid<<<sblocks(3LL * n, 256), 256, 0, st>>>(s.F32, c.fx, 3 * n, s.E3, s.scratch);
    const float kappa = (float)(s.w_force / (3.0 * n * s.force_var));
    k_sg_ctrans<<<sblocks(n, 4), 128, 0, st>>>(c.pos, n, c.sl, c.slen, c.box, s.P, s.E3,
                                                 -2.f * kappa * gsc, s.istd_d, s.V);
    cudaMemsetAsync(s.FG_d, 0, sizeof(float) * s.fh_np, st);
    fh_backward(s, s.V, n, st);
    s.fh_step++;
    k_adam_n<<<sblocks(s.fh_np, 256), 256, 0, st>>>(s.FP_d, s.FM_d, s.FV_d, s.FG_d, s.fh_np,
                                                    s.fh_step, lr, 0.9f, 0.999f, 1e-8f);
    if (it >= steps - std::min(steps, 2 * ncfg)) {  // loss over the last pass
      double lf[2];
      cudaMemcpyAsync(lf, s.scratch, sizeof(double) * 2, cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
      acc_f += lf[0] / (3.0 * n * s.force_var);
      nacc++;
    }
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  s.last_loss_e = 0.0;
  s.last_loss_f = nacc ? acc_f / nacc : 0.0;
  if (loss_e) *loss_e = 0.0;
  if (loss_f) *loss_f = s.last_loss_f;
  return (int)cudaGetLastError();
}
}  // namespace

namespace {
// the descriptor range of the stored configurations (normalised), widened
// by range_margin of each feature's span
int fm_range(Surrogate& s, cudaStream_t st) {
  cudaError_t e;
  long long h = 0;
  if (!s.xlo_d) {
    if ((e = sur_grow(s.xlo_d, h, 32)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.xhi_d, h, 32)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.oor_d, h, 4)) != cudaSuccess) return e;
  }
  int init[64];
  for (int f = 0; f < 32; f++) {
    init[f] = INT_MAX;
    init[32 + f] = INT_MIN;
  }
  // the ordered keys are kept in xlo_d and xhi_d until they are decoded below
  int* klo = reinterpret_cast<int*>(s.xlo_d);
  int* khi = reinterpret_cast<int*>(s.xhi_d);
  cudaMemcpyAsync(klo, init, sizeof(int) * 32, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(khi, init + 32, sizeof(int) * 32, cudaMemcpyHostToDevice, st);
  for (const SurConfig& c : s.cfgs)
    if (c.X && c.n > 0) k_feat_range<<<304, 256, 0, st>>>(c.X, 32LL * c.n, klo, khi);
  int keys[64];
  cudaMemcpyAsync(keys, klo, sizeof(int) * 32, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(keys + 32, khi, sizeof(int) * 32, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  float lo[32], hi[32];
  for (int f = 0; f < 32; f++) {
    auto val = [](int k) {
      const int b = k >= 0 ? k : k ^ 0x7FFFFFFF;
      float v;
      std::memcpy(&v, &b, sizeof(v));
      return v;
    };
    const float a = val(keys[f]), b = val(keys[32 + f]), span = b - a;
    lo[f] = a - s.range_margin * span;
    hi[f] = b + s.range_margin * span;
  }
  return sur_range(s, lo, hi, true, st);
}
}  // namespace

int sur_range(Surrogate& s, float* lo, float* hi, bool set, cudaStream_t st) {
  cudaError_t e;
  if (set) {
    long long h = 0;
    if (!s.xlo_d) {
      if ((e = sur_grow(s.xlo_d, h, 32)) != cudaSuccess) return e;
      h = 0;
      if ((e = sur_grow(s.xhi_d, h, 32)) != cudaSuccess) return e;
      h = 0;
      if ((e = sur_grow(s.oor_d, h, 4)) != cudaSuccess) return e;
    }
    cudaMemcpyAsync(s.xlo_d, lo, sizeof(float) * 32, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(s.xhi_d, hi, sizeof(float) * 32, cudaMemcpyHostToDevice, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    s.have_range = true;
    return 0;
  }
  if (!s.have_range) return -1;
  cudaMemcpyAsync(lo, s.xlo_d, sizeof(float) * 32, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hi, s.xhi_d, sizeof(float) * 32, cudaMemcpyDeviceToHost, st);
  return cudaStreamSynchronize(st);
}

int sur_train_fm(Surrogate& s, int steps, float lr, double* loss_e, double* loss_f,
                 cudaStream_t st) {
  if (s.cfgs.empty()) return -1;
  cudaError_t e;
  set_attrs();
  if (!s.normalised) {
    int r = sur_normalise_cfgs(s, st);
    if (r) return r;
  }
  int nmax = 0;
  for (SurConfig& c : s.cfgs) {
    nmax = std::max(nmax, c.n);
    if (!c.X) {
      if ((e = cudaMalloc(&c.X, sizeof(float) * kDesc * c.n)) != cudaSuccess) return e;
      if ((e = cudaMalloc(&c.T, sizeof(float) * c.n)) != cudaSuccess) return e;
      k_normalise<<<sblocks(c.n, 256), 256, 0, st>>>(c.G, c.eatom, c.n, s.mean_d, s.istd_d,
                                                     s.mu, s.sigma, c.X, c.T);
    }
  }
  // scratch of the largest configuration
  if (nmax > s.n_alloc) {
    long long h;
    for (float** p : {&s.dtdx, &s.gcoef}) {
      h = 0;
      if ((e = sur_grow(*p, h, (long long)nmax * kDesc)) != cudaSuccess) return e;
    }
    h = 0;
    if ((e = sur_grow(s.t, h, nmax)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.F32, h, 3LL * nmax)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.eatom, h, nmax)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.X, h, (long long)nmax * kDesc)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.slen, h, nmax)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.pos32, h, nmax)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.sl, h, (long long)nmax * kSgMax)) != cudaSuccess) return e;
    s.n_sl = (long long)nmax * kSgMax;
    s.n_alloc = nmax;
  }
  if (nmax > s.n_fm) {
    long long h = 0;
    if ((e = sur_grow(s.V, h, (long long)nmax * kDesc)) != cudaSuccess) return e;
    h = 0;
    if ((e = sur_grow(s.E3, h, 3LL * nmax)) != cudaSuccess) return e;
    s.n_fm = nmax;
  }
  if (nmax > s.n_iota) {
    std::vector<int> io(nmax);
    for (int k = 0; k < nmax; k++) io[k] = k;
    long long h = 0;
    if ((e = sur_grow(s.iota_d, h, nmax)) != cudaSuccess) return e;
    cudaMemcpyAsync(s.iota_d, io.data(), sizeof(int) * nmax, cudaMemcpyHostToDevice, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    s.n_iota = nmax;
  }
  if ((e = (cudaError_t)fm_range(s, st)) != cudaSuccess) return e;
  if (s.kind == 1) return train_fh(s, steps, lr, nmax, loss_e, loss_f, st);
  const NetDev w = net_of(s);
  double acc_e = 0, acc_f = 0;
  int nacc = 0;
  const int ncfg = (int)s.cfgs.size();
  for (int it = 0; it < steps; it++) {
    const SurConfig& c = s.cfgs[(it * 7919 + (int)(s.seed % 101)) % ncfg];
    const int n = c.n;
    const int tiles = (n + 127) / 128;
    // forces of the current network on this configuration
    k_net_infer<<<tiles, 128, kSmInfer, st>>>(c.X, n, w, s.t, s.dtdx, s.status_d);
    k_sg_scale<<<sblocks(n, 256), 256, 0, st>>>(s.t, s.dtdx, n, s.mu, s.sigma, s.istd_d,
                                                s.gcoef, s.eatom);
    cudaMemsetAsync(s.F32, 0, sizeof(float) * 3 * (size_t)n, st);
    k_sg_force<<<sblocks(n, 4), 128, 0, st>>>(c.pos, n, c.sl, c.slen, c.box, s.P, s.gcoef,
                                                s.F32);
    cudaMemsetAsync(s.scratch, 0, sizeof(double) * 2, st);
    k_fm_resid<<<sblocks(3LL * n, 256), 256, 0, st>>>(s.F32, c.fx, 3 * n, s.E3, s.scratch);
    // dL_F/d(dt/dx) = -2 kappa sigma istd q with kappa = w_force / (3 n var_F)
    const float kappa = (float)(s.w_force / (3.0 * n * s.force_var));
    k_sg_ctrans<<<sblocks(n, 4), 128, 0, st>>>(c.pos, n, c.sl, c.slen, c.box, s.P, s.E3,
                                                 (float)(-2.0 * kappa * s.sigma), s.istd_d, s.V);
    cudaMemsetAsync(s.G_d, 0, sizeof(float) * kParams, st);
    cudaMemsetAsync(s.loss_d, 0, sizeof(double), st);
    if (s.w_energy > 0.f)
      k_net_train<<<tiles, 128, kSmTrain, st>>>(c.X, c.T, n, s.iota_d, n, 0ULL, w,
                                                s.w_energy / (float)n, s.G_d, s.loss_d,
                                                s.status_d);
    if (s.w_force > 0.f)
      k_net_train_force<<<tiles, 128, kSmForce, st>>>(c.X, s.V, n, w, s.G_d, s.status_d);
    s.adam_step++;
    k_adam<<<sblocks(kParams, 256), 256, 0, st>>>(s.P_d, s.M_d, s.V_d, s.G_d, s.adam_step, lr,
                                                 0.9f, 0.999f, 1e-8f);
    k_net_cast<<<sblocks(kHid * kHid, 256), 256, 0, st>>>(s.P_d, s.W1, s.W1T, s.W2, s.W2T);
    if (it >= steps - std::min(steps, 2 * ncfg)) {  // losses over the last pass
      double le = 0, lf[2];
      cudaMemcpyAsync(&le, s.loss_d, sizeof(double), cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(lf, s.scratch, sizeof(double) * 2, cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
      acc_e += s.w_energy > 0.f ? le / s.w_energy : 0.0;
      acc_f += lf[0] / (3.0 * n * s.force_var);
      nacc++;
    }
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  s.last_loss_e = nacc ? acc_e / nacc : 0.0;
  s.last_loss_f = nacc ? acc_f / nacc : 0.0;
  if (loss_e) *loss_e = s.last_loss_e;
  if (loss_f) *loss_f = s.last_loss_f;
  return (int)cudaGetLastError();
}

int sur_force_grad(Surrogate& s, const float* X, const float* V, int n, float* grad,
                   cudaStream_t st) {
  cudaError_t e;
  set_attrs();
  float *dX = nullptr, *dV = nullptr;
  if ((e = cudaMalloc(&dX, sizeof(float) * kDesc * n)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&dV, sizeof(float) * kDesc * n)) != cudaSuccess) {
    cudaFree(dX);
    return e;
  }
  cudaMemcpyAsync(dX, X, sizeof(float) * kDesc * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dV, V, sizeof(float) * kDesc * n, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(s.G_d, 0, sizeof(float) * kParams, st);
  k_net_train_force<<<(n + 127) / 128, 128, kSmForce, st>>>(dX, dV, n, net_of(s), s.G_d,
                                                           s.status_d);
  cudaMemcpyAsync(grad, s.G_d, sizeof(float) * kParams, cudaMemcpyDeviceToHost, st);
  e = cudaStreamSynchronize(st);
  cudaFree(dX);
  cudaFree(dV);
  if (e != cudaSuccess) return e;
  return (int)cudaGetLastError();
}

int sur_rel_err(const double* a, const double* b, int n, double* scratch, double* err,
                cudaStream_t st) {
  cudaMemsetAsync(scratch, 0, sizeof(double) * 2, st);
  k_err2<<<std::max(1, std::min(256, sblocks(3LL * n, 256))), 256, 0, st>>>(a, b, 3 * n, scratch);
  double h[2];
  cudaError_t e = cudaMemcpyAsync(h, scratch, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  *err = h[1] > 0 ? sqrt(h[0] / h[1]) : 0.0;
  return 0;
}

}  // namespace mdgb

md_surrogate::~md_surrogate() {
  void* ptrs[] = {P_d, M_d,   V_d, G_d,   W1,    W1T,     W2,     W2T,    mean_d, istd_d,
                  sl,  slen,  X,   t,     dtdx,  gcoef,   F32,    eatom,  SG,     SE,
                  SX,  ST,    loss_d, scratch, rows_d, Xg, Tg, status_d};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (void* p : {(void*)iota_d, (void*)V, (void*)E3, (void*)pos32})
    if (p) cudaFree(p);
  for (void* p : {(void*)xlo_d, (void*)xhi_d, (void*)oor_d})
    if (p) cudaFree(p);
  for (void* p : {(void*)FP_d, (void*)FM_d, (void*)FV_d, (void*)FG_d, (void*)fh_gs,
                  (void*)fh_xT, (void*)fh_h1T, (void*)fh_h2T, (void*)fh_d1T, (void*)fh_d2T,
                  (void*)fh_d3T})
    if (p) cudaFree(p);
  for (mdgb::SurConfig& c : cfgs)
    for (void* p : {(void*)c.pos, (void*)c.sl, (void*)c.slen, (void*)c.fx, (void*)c.eatom,
                    (void*)c.G, (void*)c.X, (void*)c.T})
      if (p) cudaFree(p);
  if (stream) cudaStreamDestroy(stream);
}

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
