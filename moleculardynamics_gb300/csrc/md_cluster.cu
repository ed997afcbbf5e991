// Cell-cluster neighbour build and the shared-memory-staged FP32 LJ force of
// the precision form in periodic boxes (md_cluster.h has the layout).
//
// Build, per list rebuild (replaces common/NeighborList.cpp:14-156 for the
// periodic precision form; cell arithmetic as md_neighbor.cu's periodic grid):
//   1. wrap each position into its box and find its dense cell; count;
//   2. exclusive scan of the counts; scatter; rank each cell's atoms by
//      original index; permute the state into that order;
//   3. cut every z-column greedily into segments of at most one block of
//      atoms; per segment, the staged pieces of its 9 neighbour columns;
//   4. per atom, the compact row: staged offsets of the candidates within
//      the list radius, in candidate order (counted, then written).
// Force: one block per segment stages its neighbourhood (FP32 positions with
// periodic images applied) while TMA streams the segment's rows in tiles of
// 16 slots (double-buffered, mbarrier-completed); every atom of the segment
// then walks its compact row against shared memory.  Pair arithmetic and the
// cutoff band rule are those of md_forces.cu's FP32 kernels.  When the skin
// flag is up, the block walks full candidate rows from shared memory and
// refreshes the compact rows.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "md_cluster.h"
#include "md_gear.cuh"
#include "md_neighbor.cuh"
#include "md_potential.cuh"
#include "md_tma.cuh"

namespace mdgb {

cudaError_t scan_exclusive(const int* in, int* out, int n, Scratch& sc, cudaStream_t st);

namespace {

constexpr int kOffW = kClusterMaxZ + 3;  // z slots of the per-segment offset table

// replica holding atom / cell / column i (the *0 fields ascend)
template <int ClusterReplica::*F>
__device__ __forceinline__ int find_rep(const ClusterReplica* reps, int nrep, int i) {
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (reps[mid].*F <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__host__ __device__ __forceinline__ int cid(const ClusterReplica& r, int cx, int cy, int cz) {
  return r.cell0 + (cx * r.G + cy) * r.G + cz;
}

__device__ __forceinline__ int wrapc(int c, int G, int& img) {
  img = 0;
  if (c < 0) { c += G; img = -1; }
  if (c >= G) { c -= G; img = 1; }
  return c;
}

__device__ __forceinline__ int zimg(int z, int G) { return z < 0 ? -1 : (z >= G ? 1 : 0); }

// 1. wrap into [-L/2, L/2) and find the dense cell (the arithmetic of
// md_neighbor.cu's periodic grid: x - L floor((x + L/2) / L), then
// (int)((x + L/2) / cs) clamped to the grid); count atoms per cell
__global__ void k_cl_assign(md_double4* __restrict__ pos, int n, const ClusterReplica* reps,
                            int nrep, int* __restrict__ cell, int* __restrict__ count,
                            int* __restrict__ counters, int* __restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ClusterReplica r = reps[find_rep<&ClusterReplica::atom0>(reps, nrep, i)];
  md_double4 p = pos[i];
  double x[3] = {p.x, p.y, p.z};
  const double h = r.L * 0.5;
  int c[3];
  bool bad = false;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    // floor((x + h) / L) and trunc((x + h) / cs) with the exact divisions,
    // which GB300's narrow FP64 pipe makes costly: a product with the
    // reciprocal (within 2 ulp of the quotient) decides unless the quotient
    // lies within 1e-12 of an integer
    const double xa = xadd(x[d], h);
    double q = 0.0;  // 0 <= x + L/2 < L: the rounded quotient lies in [0, 1)
    if (!(xa >= 0.0 && xa < r.L)) {
      const double qa = xa * r.invL;
      q = fabs(qa - rint(qa)) > 1e-12 * fmax(1.0, fabs(qa)) ? floor(qa) : floor(xdiv(xa, r.L));
      x[d] = xsub(x[d], xmul(q, r.L));
    }
    const double xb = q == 0.0 ? xa : xadd(x[d], h);
    const double sa = xb * r.invcs;
    double s = fabs(sa - rint(sa)) > 1e-12 * fmax(1.0, fabs(sa)) ? sa : xdiv(xb, r.cs);
    if (!(s >= 0.0 && s < 2.0e9)) {
      bad = true;
      s = 0.0;
    }
    const int cc = __double2int_rz(s);
    c[d] = cc >= r.G ? r.G - 1 : cc;
  }
  if (bad) atomicOr(status, ST_NONFINITE);
  p.x = x[0];
  p.y = x[1];
  p.z = x[2];
  pos[i] = p;
  const int id = r.G == 1 ? r.cell0 : cid(r, c[0], c[1], c[2]);
  cell[i] = id;
  const int old = atomicAdd(&count[id], 1);
  // largest cell population: one atomic per warp
  const unsigned m = __activemask();
  const unsigned big = __reduce_max_sync(m, (unsigned)(old + 1));
  if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicMax(&counters[4], (int)big);
}

__global__ void k_cl_scatter(const int* __restrict__ cell, int n, const int* __restrict__ start,
                             int* __restrict__ fill, int* __restrict__ unsorted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell[i];
  unsorted[start[c] + atomicAdd(&fill[c], 1)] = i;
}

// members of each cell in ascending original index
__global__ void k_cl_rank(const int* __restrict__ unsorted, const int* __restrict__ cell,
                          const int* __restrict__ orig, int n, const int* __restrict__ start,
                          int* __restrict__ perm) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int a = unsorted[q];
  const int c = cell[a];
  const int lo = start[c], hi = start[c + 1];
  const int key = orig[a];
  int rank = 0;
  for (int k = lo; k < hi; k++) rank += orig[unsorted[k]] < key;
  perm[lo + rank] = a;
}

template <typename T>
__global__ void k_gather(const T* __restrict__ src, T* __restrict__ dst,
                         const int* __restrict__ perm, int n) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) dst[p] = src[perm[p]];
}

__global__ void k_gather3(const double* __restrict__ src, double* __restrict__ dst,
                          const int* __restrict__ perm, int n) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int a = perm[p];
#pragma unroll
  for (int d = 0; d < 3; d++) dst[3 * p + d] = src[3 * a + d];
}

__global__ void k_cl_posf(const md_double4* __restrict__ pos, float4* __restrict__ pb,
                          float4* __restrict__ posf, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const md_double4 p = pos[i];
  const float4 v = make_float4((float)p.x, (float)p.y, (float)p.z, __int_as_float((int)p.w));
  pb[i] = v;
  posf[i] = v;
}

// 3a. greedy cut of each z-column: a segment starts at z = 0 and wherever
// the next cell would take it past `cap_atoms` own atoms, `cap_staged`
// staged atoms (its 9 neighbour columns over cz0-1 .. cz1+1) or `zmax` cells
__global__ void k_seg_flags(const ClusterReplica* __restrict__ reps, int nrep, int ncols,
                            int ncells, const int* __restrict__ count, int* __restrict__ flag,
                            int cap_atoms, int cap_staged, int zmax) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col == 0) flag[ncells] = 0;
  if (col >= ncols) return;
  const ClusterReplica r = reps[find_rep<&ClusterReplica::col0>(reps, nrep, col)];
  if (r.G == 1) {
    flag[r.cell0] = 1;
    return;
  }
  const int G = r.G;
  const int local = col - r.col0;
  const int cx = local / G, cy = local % G;
  int nbase[9];  // first cell of each neighbour column
  for (int g = 0; g < 9; g++) {
    int ix, iy;
    nbase[g] = cid(r, wrapc(cx + g / 3 - 1, G, ix), wrapc(cy + g % 3 - 1, G, iy), 0);
  }
  // atoms of the 9 neighbour columns at z (periodic in z)
  auto layer = [&](int z) {
    z = z < 0 ? z + G : (z >= G ? z - G : z);
    int s = 0;
    for (int g = 0; g < 9; g++) s += count[nbase[g] + z];
    return s;
  };
  const int base = nbase[4];
  int acc = 0, cells = 0, staged = 0;
  for (int z = 0; z < G; z++) {
    const int c = count[base + z];
    const bool cut = z == 0 || cells == zmax || (acc > 0 && acc + c > cap_atoms) ||
                     staged + layer(z + 1) > cap_staged;
    flag[base + z] = cut ? 1 : 0;
    if (cut) {
      acc = c;
      cells = 1;
      staged = layer(z - 1) + layer(z) + layer(z + 1);
    } else {
      acc += c;
      cells++;
      staged += layer(z + 1);
    }
  }
}

// 3b. segment geometry at its scanned index
__global__ void k_seg_emit(const ClusterReplica* __restrict__ reps, int nrep, int ncells,
                           const int* __restrict__ flag, const int* __restrict__ segidx,
                           ClusterSegment* __restrict__ seg) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells || !flag[c]) return;
  const int k = find_rep<&ClusterReplica::cell0>(reps, nrep, c);
  const ClusterReplica r = reps[k];
  ClusterSegment& S = seg[segidx[c]];
  S.rep = k;
  if (r.G == 1) {
    S.cx = S.cy = S.cz0 = S.cz1 = 0;
    return;
  }
  const int local = c - r.cell0;
  const int cz = local % r.G;
  int z = cz + 1;
  while (z < r.G && !flag[c - cz + z]) z++;
  S.cx = local / (r.G * r.G);
  S.cy = (local / r.G) % r.G;
  S.cz0 = cz;
  S.cz1 = z - 1;
}

// 3c. pieces of each segment: for each (dx, dy) group the z range
// cz0-1 .. cz1+1, split where the periodic image changes
__global__ void k_cl_segments(ClusterSegment* __restrict__ seg, const int* __restrict__ nseg_dev,
                              const ClusterReplica* __restrict__ reps,
                              const int* __restrict__ start, int* __restrict__ counters) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= *nseg_dev) return;
  ClusterSegment& S = seg[s];
  const ClusterReplica r = reps[S.rep];
  if (r.G == 1) {
    ClusterPiece pc;
    pc.src = start[r.cell0];
    pc.count = start[r.cell0 + 1] - pc.src;
    pc.dst = 0;
    pc.ix = pc.iy = pc.iz = pc.pad = 0;
    S.p0 = pc.src;
    S.p1 = pc.src + pc.count;
    S.piece[0] = pc;
    for (int g = 0; g < 10; g++) S.group[g] = g == 9 ? 1 : 0;
    S.npieces = 1;
    S.staged = pc.count;
    S.self0 = 0;
    S.img = 0;
    atomicMax(&counters[0], S.staged);
    return;
  }
  const int G = r.G;
  S.p0 = start[cid(r, S.cx, S.cy, S.cz0)];
  S.p1 = start[cid(r, S.cx, S.cy, S.cz1) + 1];
  int np = 0, dst = 0;
  for (int dx = -1; dx < 2; dx++)
    for (int dy = -1; dy < 2; dy++) {
      S.group[(dx + 1) * 3 + (dy + 1)] = np;
      int ix, iy;
      const int cx = wrapc(S.cx + dx, G, ix), cy = wrapc(S.cy + dy, G, iy);
      const int zend = S.cz1 + 1;
      for (int z = S.cz0 - 1; z <= zend;) {
        const int iz = zimg(z, G);
        int zb = z;
        while (zb + 1 <= zend && zimg(zb + 1, G) == iz) zb++;
        ClusterPiece pc;
        pc.src = start[cid(r, cx, cy, z - iz * G)];
        pc.count = start[cid(r, cx, cy, zb - iz * G) + 1] - pc.src;
        pc.dst = dst;
        pc.ix = (signed char)ix;
        pc.iy = (signed char)iy;
        pc.iz = (signed char)iz;
        pc.pad = 0;
        S.piece[np++] = pc;
        dst += pc.count;
        z = zb + 1;
      }
    }
  S.group[9] = np;
  S.npieces = np;
  S.staged = dst;
  // own cells cz0..cz1 lie in the image-free piece of the (0, 0) group
  int s0 = 0, img = 0;
  for (int k = 0; k < np; k++) {
    const ClusterPiece& pc = S.piece[k];
    if (k >= S.group[4] && k < S.group[5] && pc.iz == 0) s0 = pc.dst + (S.p0 - pc.src);
    img |= pc.ix | pc.iy | pc.iz;
  }
  S.self0 = s0;
  S.img = img != 0;
  atomicMax(&counters[0], dst);
}

// ---- per-block segment context in shared memory ----
struct SegShared {
  ClusterSegment S;
  ClusterReplica r;
  int self0;          // staged offset of the segment's first own atom
  int off[9][kOffW];  // staged offset of z slot w (cell cz0-1+w) of each group; w = zspan: end
};

__device__ __forceinline__ void load_segment(SegShared& sh, const ClusterSegment* seg,
                                             const ClusterReplica* reps, int sidx) {
  const int* src = (const int*)&seg[sidx];
  int* dst = (int*)&sh.S;
  for (int k = threadIdx.x; k < (int)(sizeof(ClusterSegment) / 4); k += blockDim.x)
    dst[k] = src[k];
  __syncthreads();
  const int* rs = (const int*)&reps[sh.S.rep];
  int* rd = (int*)&sh.r;
  for (int k = threadIdx.x; k < (int)(sizeof(ClusterReplica) / 4); k += blockDim.x) rd[k] = rs[k];
  if (threadIdx.x == 0) sh.self0 = sh.S.self0;  // computed at the build (k_cl_segments)
}

// staged copy of positions with the pieces' periodic images applied
__device__ __forceinline__ void stage(const SegShared& sh, const float4* __restrict__ src,
                                      float4* st) {
  const ClusterSegment& S = sh.S;
  const float Lf = sh.r.Lf, Llo = sh.r.Llo;
  for (int k = 0; k < S.npieces; k++) {
    const ClusterPiece pc = S.piece[k];
    const float sx = (float)pc.ix, sy = (float)pc.iy, sz = (float)pc.iz;
    const bool img = (pc.ix | pc.iy | pc.iz) != 0;
    for (int q = threadIdx.x; q < pc.count; q += blockDim.x) {
      float4 v = src[pc.src + q];
      if (img) {
        v.x = fmaf(sx, Lf, v.x) + sx * Llo;
        v.y = fmaf(sy, Lf, v.y) + sy * Llo;
        v.z = fmaf(sz, Lf, v.z) + sz * Llo;
      }
      st[pc.dst + q] = v;
    }
  }
}

// The same staging by bulk copies: thread 0 issues one cp.async.bulk per
// piece, all completing on `bar` (phase `parity`); after the wait the image pieces
// are shifted in place.  Returns false (uniformly) if the bounded wait ran
// out; the caller then leaves after the copies land or time out.
__device__ __forceinline__ bool stage_bulk(const SegShared& sh, const float4* __restrict__ src,
                                           float4* st, uint64_t* bar, uint32_t parity,
                                           int* status, int limit) {
  const ClusterSegment& S = sh.S;
  if (threadIdx.x < 32) {
    // one lane announces the bytes, then up to 27 lanes issue a piece each
    if (threadIdx.x == 0) {
      fence_proxy_async();  // earlier generic accesses to the stage come first
      mbar_expect_tx(bar, (uint32_t)S.staged * (uint32_t)sizeof(float4));
    }
    __syncwarp();
    const int k = threadIdx.x;
    if (k < S.npieces) {
      const ClusterPiece& pc = S.piece[k];
      if (pc.count > 0)
        bulk_load(st + pc.dst, src + pc.src, (uint32_t)pc.count * (uint32_t)sizeof(float4), bar);
    }
  }
  // the warps sleep in the wait (suspend-time hint) rather than spin
  const bool got = mbar_wait_sleep(bar, parity, status, limit);
  if (!__syncthreads_and(got)) {
    if (threadIdx.x == 0) mbar_drain(bar, parity, status);
    return false;
  }
  if (!S.img) return true;
  const float Lf = sh.r.Lf, Llo = sh.r.Llo;
  for (int k = 0; k < S.npieces; k++) {
    const ClusterPiece& pc = S.piece[k];
    if ((pc.ix | pc.iy | pc.iz) == 0) continue;
    const float sx = (float)pc.ix, sy = (float)pc.iy, sz = (float)pc.iz;
    for (int q = threadIdx.x; q < pc.count; q += blockDim.x) {
      float4 v = st[pc.dst + q];
      v.x = fmaf(sx, Lf, v.x) + sx * Llo;
      v.y = fmaf(sy, Lf, v.y) + sy * Llo;
      v.z = fmaf(sz, Lf, v.z) + sz * Llo;
      st[pc.dst + q] = v;
    }
  }
  return true;
}

__device__ __forceinline__ void fill_offsets(SegShared& sh, const int* __restrict__ start) {
  const ClusterSegment& S = sh.S;
  const ClusterReplica& r = sh.r;
  if (r.G == 1) return;
  const int zspan = S.cz1 - S.cz0 + 3;
  for (int k = threadIdx.x; k < 9 * (zspan + 1); k += blockDim.x) {
    const int g = k / (zspan + 1), w = k % (zspan + 1);
    const int pe = S.group[g + 1];
    int v;
    if (w == zspan) {
      v = S.piece[pe - 1].dst + S.piece[pe - 1].count;
    } else {
      int ix, iy;
      const int cx = wrapc(S.cx + g / 3 - 1, r.G, ix), cy = wrapc(S.cy + g % 3 - 1, r.G, iy);
      const int z = S.cz0 - 1 + w, iz = zimg(z, r.G);
      v = 0;
      for (int p = S.group[g]; p < pe; p++)
        if (S.piece[p].iz == iz) {
          v = S.piece[p].dst + (start[cid(r, cx, cy, z - iz * r.G)] - S.piece[p].src);
          break;
        }
    }
    sh.off[g][w] = v;
  }
}

// staged offset of the segment's own atom p
__device__ __forceinline__ int self_offset(const SegShared& sh, int p) {
  return sh.self0 + (p - sh.S.p0);
}

// visit(q) for every staged candidate of atom p's 27-cell row, in row order
template <typename F>
__device__ __forceinline__ void walk_staged(const SegShared& sh, int self, F&& visit) {
  if (sh.r.G == 1) {
    for (int q = 0; q < sh.S.staged; q++)
      if (q != self) visit(q);
    return;
  }
  const int zspan = sh.S.cz1 - sh.S.cz0 + 3;
  int w = 1;
  while (w < zspan - 2 && sh.off[4][w + 1] <= self) w++;
  const int u = w - 1;
  for (int g = 0; g < 9; g++) {
    const int a = sh.off[g][u], b = sh.off[g][u + 3];
    for (int q = a; q < b; q++)
      if (q != self) visit(q);
  }
}

// staged offset -> (sorted index, image)
__device__ __forceinline__ int staged_source(const ClusterSegment& S, int q, int& ix, int& iy,
                                             int& iz) {
  for (int k = 0; k < S.npieces; k++) {
    const ClusterPiece& pc = S.piece[k];
    if (q >= pc.dst && q < pc.dst + pc.count) {
      ix = pc.ix;
      iy = pc.iy;
      iz = pc.iz;
      return pc.src + (q - pc.dst);
    }
  }
  ix = iy = iz = 0;
  return S.p0;
}

__device__ __forceinline__ float min_img(float d, float Lf, float invL) {
  return d - Lf * rintf(d * invL);
}

// Rows are padded with the segment's sentinel (staged entry `staged`, a
// position far outside every cutoff) up to the longest row of the warp
// rounded up to whole 16-slot tiles, so the force loop reads only real or
// sentinel entries and needs no per-slot validity test.  Warp-collective.
__device__ __forceinline__ void pad_rows(uint16_t* __restrict__ rows, int ld, int cap, int p,
                                         bool live, int kept, int sentinel) {
  int wm = live ? min(kept, cap) : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) wm = max(wm, __shfl_xor_sync(0xffffffffu, wm, o));
  const int padded = min((wm + kClusterTileSlots - 1) / kClusterTileSlots * kClusterTileSlots, cap);
  if (live)
    for (int k = min(kept, cap); k < padded; k++) rows[(size_t)k * ld + p] = (uint16_t)sentinel;
}

// Grouped rows (the register-prefetch scheme): slots k of atom p in groups
// of eight, one 16-byte word per atom and group, rows[((k / 8) ld + p) 8 +
// k % 8], each entry the staged atom's byte offset 16 q (staged
// neighbourhoods below 4,095 atoms), so that the force loop fetches eight
// slots with one load and addresses the staged position without arithmetic.
// Otherwise slot-major staged indices, rows[k ld + p].
__device__ __forceinline__ size_t row_slot(int k, int p, int ld, int grouped) {
  return grouped ? (((size_t)(k >> 3) * ld + p) << 3) + (k & 7) : (size_t)k * ld + p;
}
__device__ __forceinline__ uint16_t row_val(int q, int grouped) {
  return (uint16_t)(grouped ? q << 4 : q);
}

// word k (0..7) of a row chunk held in registers, without indexing the
// array at run time (which would place it in local memory)
__device__ __forceinline__ uint32_t pick8(const uint32_t (&c)[8], int k) {
  const uint32_t a = (k & 1) ? c[1] : c[0], b = (k & 1) ? c[3] : c[2];
  const uint32_t d = (k & 1) ? c[5] : c[4], e = (k & 1) ? c[7] : c[6];
  const uint32_t lo = (k & 2) ? b : a, hi = (k & 2) ? e : d;
  return (k & 4) ? hi : lo;
}

// Appends a thread's grouped row entries eight at a time: entries shift into
// a 128-bit register word from the top (funnel shifts), and every full word
// is stored with one 16-byte store.  Entries past cap are counted, not stored.
struct GroupWriter {
  uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
  int n = 0;  // entries pushed
  __device__ __forceinline__ void push(uint16_t* rows, int ld, int cap, int p, uint32_t e) {
    w0 = __funnelshift_r(w0, w1, 16);
    w1 = __funnelshift_r(w1, w2, 16);
    w2 = __funnelshift_r(w2, w3, 16);
    w3 = (w3 >> 16) | (e << 16);
    ++n;
    if ((n & 7) == 0 && n <= cap)
      reinterpret_cast<uint4*>(rows)[(size_t)((n >> 3) - 1) * ld + p] = make_uint4(w0, w1, w2, w3);
  }
  // pads with the sentinel to `padded` slots (a multiple of 16, <= cap)
  __device__ __forceinline__ void finish(uint16_t* rows, int ld, int cap, int p, int padded,
                                         uint32_t sentinel) {
    while ((n & 7) != 0 && n < padded) push(rows, ld, cap, p, sentinel);
    const uint32_t s2 = sentinel | (sentinel << 16);
    for (int g = (n + 7) >> 3; 8 * g < padded; g++)
      reinterpret_cast<uint4*>(rows)[(size_t)g * ld + p] = make_uint4(s2, s2, s2, s2);
  }
};

// warp-uniform padded length: the warp's longest kept row rounded up to
// whole 16-slot tiles, at most cap
__device__ __forceinline__ int padded_len(bool live, int kept, int cap) {
  int wm = live ? min(kept, cap) : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) wm = max(wm, __shfl_xor_sync(0xffffffffu, wm, o));
  return min((wm + kClusterTileSlots - 1) / kClusterTileSlots * kClusterTileSlots, cap);
}

// pad_rows for either layout; warp-collective
__device__ __forceinline__ void pad_rows_any(uint16_t* __restrict__ rows, int ld, int cap, int p,
                                             bool live, int kept, int sentinel, int grouped) {
  if (!grouped) {
    pad_rows(rows, ld, cap, p, live, kept, sentinel);
    return;
  }
  const int padded = padded_len(live, kept, cap);
  if (live)
    for (int k = min(kept, cap); k < padded; k++)
      rows[row_slot(k, p, ld, 1)] = row_val(sentinel, 1);
}

__device__ __forceinline__ void put_sentinel(float4* st, int staged) {
  if (threadIdx.x == 0) st[staged] = make_float4(1e18f, 1e18f, 1e18f, __int_as_float(SP_NG));
}

constexpr int kRowStep = 8;  // staged candidates tested per step of the row walk

// 4. compact rows from the build-time positions (MODE 0: count, 1: write,
// 2: both, rows longer than cap truncated and reported through the counters)
template <int MODE>
__global__ void __launch_bounds__(256)
    k_cl_rows(const ClusterSegment* __restrict__ seg, const ClusterReplica* __restrict__ reps,
              const int* __restrict__ start, const float4* __restrict__ pb, float rv2,
              uint16_t* __restrict__ rows, uint16_t* __restrict__ len, int ld, int cap,
              int* __restrict__ counters, int grouped) {
  extern __shared__ float4 st[];
  __shared__ SegShared sh;
  load_segment(sh, seg, reps, blockIdx.x);
  __syncthreads();
  stage(sh, pb, st);
  fill_offsets(sh, start);
  __syncthreads();
  const bool minimg = sh.r.G == 1;
  const float Lf = sh.r.Lf, invL = 1.0f / sh.r.Lf;
  int mx = 0;
  unsigned long long tot = 0;
  for (int base = sh.S.p0; base < sh.S.p1; base += blockDim.x) {
    const int p = base + threadIdx.x;
    const bool live = p < sh.S.p1;
    int kept = 0;
    GroupWriter gw;
    if (live && !minimg) {
      // the 9 column groups in row order, kRowStep independent distance
      // tests per step; only the centre group holds the atom itself
      const int self = self_offset(sh, p);
      const float4 pi = st[self];
      const int zspan = sh.S.cz1 - sh.S.cz0 + 3;
      int w = 1;
      while (w < zspan - 2 && sh.off[4][w + 1] <= self) w++;
      const int u = w - 1;
      auto near = [&](int q) {
        const float4 pj = st[q];
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        return dx * dx + dy * dy + dz * dz < rv2;
      };
      auto take = [&](int q, bool in) {
        if (in) {
          if (MODE != 0) {
            if (grouped)
              gw.push(rows, ld, cap, p, (uint32_t)q << 4);
            else if (kept < cap)
              rows[(size_t)kept * ld + p] = (uint16_t)q;
          }
          kept++;
        }
      };
      auto group = [&](int g, auto centre) {
        const int qa = sh.off[g][u], qb = sh.off[g][u + 3];
        int q = qa;
        for (; q + kRowStep <= qb; q += kRowStep) {
          bool in[kRowStep];
#pragma unroll
          for (int u = 0; u < kRowStep; u++)
            in[u] = near(q + u) && (!decltype(centre)::value || q + u != self);
#pragma unroll
          for (int u = 0; u < kRowStep; u++) take(q + u, in[u]);
        }
        for (; q < qb; q++) take(q, near(q) && (!decltype(centre)::value || q != self));
      };
#pragma unroll 1
      for (int g = 0; g < 4; g++) group(g, std::false_type());
      group(4, std::true_type());
#pragma unroll 1
      for (int g = 5; g < 9; g++) group(g, std::false_type());
    } else if (live) {
      const int self = self_offset(sh, p);
      const float4 pi = st[self];
      walk_staged(sh, self, [&](int q) {
        const float4 pj = st[q];
        float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        if (minimg) {
          dx = min_img(dx, Lf, invL);
          dy = min_img(dy, Lf, invL);
          dz = min_img(dz, Lf, invL);
        }
        if (dx * dx + dy * dy + dz * dz < rv2) {
          if (MODE != 0) {
            if (grouped)
              gw.push(rows, ld, cap, p, (uint32_t)q << 4);
            else if (kept < cap)
              rows[(size_t)kept * ld + p] = (uint16_t)q;
          }
          kept++;
        }
      });
    }
    if (MODE != 0) {
      if (grouped) {
        const int padded = padded_len(live, kept, cap);
        if (live) gw.finish(rows, ld, cap, p, padded, (uint32_t)sh.S.staged << 4);
      } else {
        pad_rows(rows, ld, cap, p, live, kept, sh.S.staged);
      }
    }
    if (MODE != 1 && live) {
      len[p] = (uint16_t)min(kept, 65535);
      mx = max(mx, kept);
      tot += (unsigned long long)kept;
    }
  }
  if (MODE != 1) {
    // one atomic per warp (all threads of the block reach this point)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&counters[1], mx);
      atomicAdd((unsigned long long*)(counters + 2), tot);
    }
  }
}

__device__ __forceinline__ void kahan_add(float& hi, float& lo, float x) {
  const float y = x - lo;
  const float t = hi + y;
  lo = (t - hi) - y;
  hi = t;
}

template <int NV>
__device__ __forceinline__ void block_sums(double (&v)[NV], double* out) {
  __shared__ double sm[NV][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sm[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0;
    for (int w = 0; w < nw; w++) s += sm[threadIdx.x][w];
    out[NV * blockIdx.x + threadIdx.x] = s;
  }
}

// block sum of NV doubles into out[NV * slot + k]
template <int NV>
__device__ __forceinline__ void block_sums_at(double (&v)[NV], double* out, int slot) {
  __shared__ double sm[NV][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sm[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0;
    for (int w = 0; w < nw; w++) s += sm[threadIdx.x][w];
    out[NV * slot + threadIdx.x] = s;
  }
}

// Pair (p, q) within 1e-5 of the cutoff: decided in FP64 as the FP64 path
// decides it (same image, same roundings).
__device__ __noinline__ bool band_inside(const SegShared& sh, const md_double4* pos, int p,
                                         int q, double rcutsq) {
  int ix, iy, iz;
  const int j = staged_source(sh.S, q, ix, iy, iz);
  const md_double4 a = pos[p], b = pos[j];
  const double L = sh.r.L;
  if (sh.r.G == 1) {
    ix = min_image(a.x, b.x, L);
    iy = min_image(a.y, b.y, L);
    iz = min_image(a.z, b.z, L);
  }
  double xj = b.x, yj = b.y, zj = b.z;
  if (ix | iy | iz) {
    xj = xadd(xj, (double)ix * L);
    yj = xadd(yj, (double)iy * L);
    zj = xadd(zj, (double)iz * L);
  }
  return norm2_exact(xsub(a.x, xj), xsub(a.y, yj), xsub(a.z, zj)) < rcutsq;
}

// LJ parameters of the force loops: one species (P, Q of the inv^4 form) or
// the three NG pair kinds (sigma^2, 24 eps)
struct LjParams {
  float s2[3], c24[3];
  float p, q;
};

// The padded-row loops decide pairs within 1e-5 of the cutoff afterwards:
// the atom's row is walked again (entries from global memory, in row order),
// and every pair in the band that the FP64 decision keeps is added, in row
// order, to one FP32 sum, folded once into the compensated force.  Rare
// (about one atom in 600 has such a pair).
template <bool ALL_NG>
__device__ __noinline__ float3 band_pass(const SegShared& sh, const float4* st,
                                         const md_double4* pos, double rcutsq,
                                         const uint16_t* rows, int ld, int grouped, int p, int L,
                                         float4 pi, float rc_lo, float rc_hi, LjParams lp) {
  float ex = 0.f, ey = 0.f, ez = 0.f;
  const int ti = __float_as_int(pi.w);
  for (int k = 0; k < L; k++) {
    const int e = rows[row_slot(k, p, ld, grouped)];
    const int q = grouped ? e >> 4 : e;
    const float4 pj = st[q];
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (!(r2 > rc_lo && r2 < rc_hi)) continue;
    float fij;
    const float inv = rcp_approx(r2);
    if (ALL_NG) {
      const float inv2 = inv * inv;
      fij = (inv2 * inv2) * fmaf(lp.p, inv2 * inv, -lp.q);
    } else {
      const int tj = __float_as_int(pj.w);
      if (!(tj == SP_NG || ti == SP_NG)) continue;
      const int sel = lj_select(ti, tj);
      const float s2 = sel == SP_N ? lp.s2[0] : (sel == SP_O ? lp.s2[1] : lp.s2[2]);
      const float c24 = sel == SP_N ? lp.c24[0] : (sel == SP_O ? lp.c24[1] : lp.c24[2]);
      const float sr2 = s2 * inv;
      const float sr6 = sr2 * sr2 * sr2;
      fij = c24 * inv * sr6 * fmaf(2.0f, sr6, -1.0f);
    }
    if (!band_inside(sh, pos, p, q, rcutsq)) continue;
    ex = fmaf(dx, fij, ex);
    ey = fmaf(dy, fij, ey);
    ez = fmaf(dz, fij, ez);
  }
  return make_float3(ex, ey, ez);
}

// Arguments of the segment force kernel (device copy of ClusterForceArgs).
struct ClStep {
  int nseg;
  int* sched;  // [0] next segment to hand out, [1] blocks finished
  const ClusterSegment* seg;
  const ClusterReplica* reps;
  const int* start;
  const float4* posf;
  const md_double4* pos;
  double* f3;
  uint16_t* rows;
  uint16_t* len;
  int ld, cap;
  float rv2;
  float4* pos_build;
  int* skin;
  int flag_read, flag_set, flag_clear;
  double rcutsq;
  Species sp;
  double* epart;
  int* status;
  ClusterGearArgs g;
  int nbuf;  // row tiles in flight in the block-tile scheme (2 or 3)
  int wait_limit;  // polls of a bounded mbarrier wait
  int grouped;     // rows grouped by eight slots, byte offsets (row_slot)
  // the lean kernel's cutoff band (rc_lo, rc_hi, rc_mid, rc_half) and LJ
  // factors (P, Q), computed on the host with k_lj_cl's float expressions:
  // as kernel parameters they need no registers in the pair loop
  float lean_c[6];
};

// FP32 LJ force, persistent: each block takes segments from a shared
// counter until none is left.  ev: E, E_shifted, W per segment (as md_forces.cu).
// GEAR 1: the Gear correct of this step and predict of the next follow for each
// atom in the same thread (cpu/common/Device.cpp:17-85 in FP64 with FMAs);
// GEAR 2: the correct only (a list build, a record or the call's end follows),
// forces also stored.
// Dynamic shared memory: two row tiles [16][blockDim + 8] of uint16 (TMA
// destinations), then the staged positions.
// Row loads: ROWS 0, tiles of the whole block by TMA into shared memory
// (block-synchronised; two or three tiles in flight); 1, each lane prefetches its next 16 entries into
// registers; 2, tiles of each warp by TMA (warp-synchronised, each warp
// walks only its own longest row)
constexpr int kWarpTileAtoms = 40;  // 32 atoms + up to 8 for the 16-byte start
constexpr int kWarpTileBytes = kWarpTileAtoms * kClusterTileSlots * 2;

template <bool ENERGY, bool ALL_NG, int GEAR, int ROWS>
__global__ void __launch_bounds__(224, 3)
    k_lj_cl(const __grid_constant__ CUtensorMap rmap, const ClStep a) {
  extern __shared__ __align__(128) unsigned char dyn[];
  const int tid = threadIdx.x;
  const int BX = blockDim.x + 8;
  uint16_t* tiles = (uint16_t*)dyn;
  const int nbuf = a.nbuf;  // block tiles in flight (ROWS 0): 2 or 3
  const uint32_t tile_elems = kClusterTileSlots * BX;
  const uint32_t tile_bytes = tile_elems * sizeof(uint16_t);
  const int tile_region =
      ROWS == 0 ? nbuf * kClusterTileSlots * BX * (int)sizeof(uint16_t)
                : (ROWS == 2 ? (int)(blockDim.x >> 5) * 2 * kWarpTileBytes : 0);
  float4* st = (float4*)(dyn + tile_region);
  __shared__ __align__(8) uint64_t wbar[7][2];  // ROWS 2: two tile barriers per warp
  __shared__ SegShared sh;
  __shared__ __align__(8) uint64_t bar[4];  // up to three row tiles, staging
  __shared__ int s_max[8];
  __shared__ int s_trip;
  if (tid == 0) {
    // an energy evaluation follows a correct-only launch of the same step,
    // which records a trip of the corrected positions in the next step's flag
    s_trip = (a.skin[a.flag_read] | a.skin[3] | (ENERGY ? a.skin[a.flag_set] : 0)) != 0;
    for (int k = 0; k < 4; k++) mbar_init(&bar[k], 1);
    if (ROWS == 2)
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        mbar_init(&wbar[w][0], 1);
        mbar_init(&wbar[w][1], 1);
      }
    fence_mbar_init();
  }
  __syncthreads();
  const bool tripped = s_trip != 0;
  uint32_t phase = 0u;       // bit b: parity to wait for on bar[b] (b = 3: staging)
  uint32_t inflight = 0u;    // bit b: a copy into buffer b is in flight (issuing thread)
  bool trip_next = false;
  bool aborted = false;
  __shared__ int s_seg;
  for (;;) {
  // segments are handed out dynamically; the last block to leave resets
  // the counters for the next launch
  if (tid == 0) s_seg = atomicAdd(&a.sched[0], 1);
  __syncthreads();
  const int sidx = s_seg;
  if (sidx >= a.nseg) break;
  load_segment(sh, a.seg, a.reps, sidx);
  __syncthreads();
  // block tiles: the segment's first two row tiles go to L2 while the
  // neighbourhood streams in (no completion to wait for)
  if (ROWS == 0 && !tripped && tid == 0) {
    tma_prefetch_2d(&rmap, sh.S.p0 & ~7, 0);
    tma_prefetch_2d(&rmap, sh.S.p0 & ~7, kClusterTileSlots);
  }
  if (!stage_bulk(sh, a.posf, st, &bar[3], (phase >> 3) & 1u, a.status, a.wait_limit)) {
    aborted = true;
    break;
  }
  phase ^= 8u;
  put_sentinel(st, sh.S.staged);
  if (tripped) fill_offsets(sh, a.start);
  __syncthreads();
  const bool minimg = sh.r.G == 1;
  // without minimum images or energies the sentinel-padded rows need no
  // per-slot validity test (the sentinel lies beyond every cutoff)
  const bool fast = !ENERGY && !minimg;
  const float Lf = sh.r.Lf, invL = 1.0f / sh.r.Lf;
  const float rc2 = (float)a.rcutsq;
  const float rc_lo = rc2 * (1.0f - 1e-5f), rc_hi = rc2 * (1.0f + 1e-5f);
  // |r2 - rc_mid| < rc_half covers (rc_lo, rc_hi) with a little to spare
  const float rc_mid = 0.5f * (rc_lo + rc_hi), rc_half = 0.5f * (rc_hi - rc_lo) * 1.001f;
  const float s2_ng = a.sp.sig[2] * a.sp.sig[2], c_ng = 24.0f * a.sp.eps[2];
  const float s2_n = a.sp.sig[0] * a.sp.sig[0], c_n = 24.0f * a.sp.eps[0];
  const float s2_o = a.sp.sig[1] * a.sp.sig[1], c_o = 24.0f * a.sp.eps[1];
  // LJ factor F/r of a pair, inv = 1/r^2.  One species (ALL_NG):
  // inv^4 (P inv^3 - Q), P = 48 eps sigma^12, Q = 24 eps sigma^6, in every
  // row scheme and in the lean kernel (so that the scheme does not change a
  // bit of the result); mixed species: 24 eps inv (sigma^2 inv)^3
  // (2 (sigma^2 inv)^3 - 1) with the pair's parameters.
  const float q6 = s2_ng * s2_ng * s2_ng;
  const float lj_q = c_ng * q6, lj_p = 2.0f * c_ng * q6 * q6;
  auto lj_factor = [&](float inv, float s2, float c24) {
    if (ALL_NG) {
      const float inv2 = inv * inv;
      return (inv2 * inv2) * fmaf(lj_p, inv2 * inv, -lj_q);
    }
    const float sr2 = s2 * inv;
    const float sr6 = sr2 * sr2 * sr2;
    return c24 * inv * sr6 * fmaf(2.0f, sr6, -1.0f);
  };
  double ev[3] = {0.0, 0.0, 0.0};
  const int p0 = sh.S.p0, p1 = sh.S.p1;
  for (int base = p0; base < p1; base += blockDim.x) {
    const int p = base + tid;
    const bool live = p < p1;
    const int self = live ? self_offset(sh, p) : 0;
    if (GEAR && live) {
      // the Gear state of this atom is read after the force loop: ask L2
      // for its lines now
      prefetch_l2(a.pos + p);
      prefetch_l2(a.g.vel + 3 * (size_t)p);
      prefetch_l2(a.g.acc + 3 * (size_t)p);
      prefetch_l2(a.g.b + 3 * (size_t)p);
      prefetch_l2(a.g.c + 3 * (size_t)p);
      prefetch_l2(a.pos_build + p);
    }
    const float4 pi = st[self];
    const int ti = __float_as_int(pi.w);
    float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
    bool band_any = false;  // a padded-row chunk had a pair in the cutoff band
    // energies (ENERGY): E, shifted E and the virial of the atom's pairs,
    // summed like the forces (FP32 within a 16-slot chunk, compensated
    // across chunks, widened to FP64 once per atom)
    float ce = 0.f, cs = 0.f, cw = 0.f;
    float eh = 0.f, el = 0.f, sh2 = 0.f, sl2 = 0.f, wh = 0.f, wl = 0.f;
    auto fold_energy = [&]() {
      if (ENERGY) {
        kahan_add(eh, el, ce);
        kahan_add(sh2, sl2, cs);
        kahan_add(wh, wl, cw);
        ce = cs = cw = 0.f;
      }
    };
    // candidate q into the running sums (cx, cy, cz); `valid` false
    // evaluates a harmless dummy (no branch)
    auto pair = [&](int q, bool valid, float& cx, float& cy, float& cz) {
      const float4 pj = st[q];
      float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      if (minimg) {
        dx = min_img(dx, Lf, invL);
        dy = min_img(dy, Lf, invL);
        dz = min_img(dz, Lf, invL);
      }
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      float s2 = s2_ng, c24 = c_ng;
      bool use = valid;
      if (!ALL_NG) {
        const int tj = __float_as_int(pj.w);
        use = use && (tj == SP_NG || ti == SP_NG);
        const int sel = lj_select(ti, tj);
        s2 = sel == SP_N ? s2_n : (sel == SP_O ? s2_o : s2_ng);
        c24 = sel == SP_N ? c_n : (sel == SP_O ? c_o : c_ng);
      }
      const float inv = rcp_approx(r2);
      const float sr2 = s2 * inv;
      const float sr6 = sr2 * sr2 * sr2;  // the energy terms below
      float fij = lj_factor(inv, s2, c24);
      bool in = r2 <= rc_lo;
      if (use && !in && r2 < rc_hi) in = band_inside(sh, a.pos, p, q, a.rcutsq);
      in = in && use;
      fij = in ? fij : 0.0f;
      cx = fmaf(dx, fij, cx);
      cy = fmaf(dy, fij, cy);
      cz = fmaf(dz, fij, cz);
      if (ENERGY) {
        const float src2 = s2 / rc2;
        const float src6 = src2 * src2 * src2;
        const float eps = c24 * (1.0f / 24.0f);
        const float e = 2.0f * eps * (sr6 * sr6 - sr6);
        ce += in ? e : 0.0f;
        cs += in ? e - 2.0f * eps * (src6 * src6 - src6) : 0.0f;
        cw += r2 * fij;  // fij is zero outside the cutoff
      }
    };
    // 16 row slots: even and odd slots in two sums (two independent FMA
    // chains), folded into the compensated sum; wrem is warp-uniform
    auto chunk16 = [&](auto&& get, int rem, int wrem) {
      float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
      if (wrem >= kClusterTileSlots) {
#pragma unroll
        for (int kk = 0; kk < kClusterTileSlots; kk += 2) {
          const bool v0 = kk < rem, v1 = kk + 1 < rem;
          const int q0 = v0 ? get(kk) : self;
          const int q1 = v1 ? get(kk + 1) : self;
          pair(q0, v0, ax, ay, az);
          pair(q1, v1, bx, by, bz);
        }
      } else {
#pragma unroll
        for (int kk = 0; kk < kClusterTileSlots; kk++) {
          if (kk < wrem) {
            const bool valid = kk < rem;
            const int q = valid ? get(kk) : self;
            if (kk & 1)
              pair(q, valid, bx, by, bz);
            else
              pair(q, valid, ax, ay, az);
          }
        }
      }
      kahan_add(hx, lx, ax + bx);
      kahan_add(hy, ly, ay + by);
      kahan_add(hz, lz, az + bz);
      fold_energy();
    };
    // The padded-row form of a pair: no validity test, and the FP64 decision
    // near the cutoff is deferred: `band` records that some pair of the
    // chunk lies within 1e-5 of it.
    auto pair_fast = [&](int q, float& cx, float& cy, float& cz, bool& band) {
      const float4 pj = st[q];
      const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      float s2 = s2_ng, c24 = c_ng;
      bool use = true;
      if (!ALL_NG) {
        const int tj = __float_as_int(pj.w);
        use = tj == SP_NG || ti == SP_NG;
        const int sel = lj_select(ti, tj);
        s2 = sel == SP_N ? s2_n : (sel == SP_O ? s2_o : s2_ng);
        c24 = sel == SP_N ? c_n : (sel == SP_O ? c_o : c_ng);
      }
      float fij = lj_factor(rcp_approx(r2), s2, c24);
      band |= use && fabsf(r2 - rc_mid) < rc_half;
      fij = use && r2 <= rc_lo ? fij : 0.0f;
      cx = fmaf(dx, fij, cx);
      cy = fmaf(dy, fij, cy);
      cz = fmaf(dz, fij, cz);
    };
    // 16 padded row slots; pairs in the band are added afterwards, each
    // decided in FP64 (rare: about one atom in 600 has one)
    auto chunk16_fast = [&](auto&& get) {
      float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
      bool band = false;
#pragma unroll
      for (int kk = 0; kk < kClusterTileSlots; kk += 2) {
        pair_fast(get(kk), ax, ay, az, band);
        pair_fast(get(kk + 1), bx, by, bz, band);
      }
      band_any |= band;  // decided after the row (band_pass)
      kahan_add(hx, lx, ax + bx);
      kahan_add(hy, ly, ay + by);
      kahan_add(hz, lz, az + bz);
    };
    int kept_new = 0;  // fresh row length of a refresh step
    if (!tripped && ROWS == 2) {
      const int warp = tid >> 5, lane = tid & 31;
      const int L = live ? (int)a.len[p] : 0;
      int wmax = L;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
      const int Tw = (wmax + kClusterTileSlots - 1) / kClusterTileSlots;
      const int wb = base + 32 * warp;
      const int x0 = wb & ~7;  // 16-byte aligned start of the warp's tile
      const int col = lane + (wb - x0);
      uint16_t* wt = (uint16_t*)(dyn + (size_t)warp * 2 * kWarpTileBytes);
      uint64_t* wb2 = wbar[warp];
      if (lane == 0) {
        for (int t = 0; t < 2 && t < Tw; t++) {
          fence_proxy_async();
          mbar_expect_tx(&wb2[t], kWarpTileBytes);
          tma_load_2d(wt + t * (kWarpTileBytes / 2), &rmap, x0, t * kClusterTileSlots, &wb2[t]);
          inflight |= 1u << t;
        }
      }
      __syncwarp();
      bool wfailed = false;
      for (int t = 0; t < Tw; t++) {
        const int b = t & 1;
        const bool got = __all_sync(
            0xffffffffu, mbar_wait(&wb2[b], (phase >> b) & 1u, a.status, a.wait_limit));
        if (!got) {
          wfailed = true;
          break;
        }
        phase ^= 1u << b;
        inflight &= ~(1u << b);
        const uint16_t* tl = wt + b * (kWarpTileBytes / 2) + col;
        auto get = [&](int kk) { return (int)tl[kk * kWarpTileAtoms]; };
        if (!fast)
          chunk16(get, L - t * kClusterTileSlots, wmax - t * kClusterTileSlots);
        else if (live)
          chunk16_fast(get);
        __syncwarp();  // the warp is done with buffer b
        if (lane == 0 && t + 2 < Tw) {
          fence_proxy_async();
          mbar_expect_tx(&wb2[b], kWarpTileBytes);
          tma_load_2d(wt + b * (kWarpTileBytes / 2), &rmap, x0, (t + 2) * kClusterTileSlots,
                      &wb2[b]);
          inflight |= 1u << b;
        }
      }
      if (!__syncthreads_and(!wfailed)) {
        // a bounded wait ran out somewhere: copies still in flight land (or
        // time out) before the block leaves
        if (lane == 0)
          for (int b = 0; b < 2; b++)
            if ((inflight >> b) & 1u) mbar_drain(&wb2[b], (phase >> b) & 1u, a.status);
        aborted = true;
        break;
      }
    } else if (!tripped && ROWS == 1) {
      // grouped rows (row_slot): each lane streams its own row, sixteen
      // slots as two 16-byte loads, one chunk in flight while the previous
      // one computes; whole padded tiles below the warp's longest row only
      // (t0 is a multiple of 16: the test is warp-uniform)
      const int L = live ? (int)a.len[p] : 0;
      int wmax = L;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
      const uint4* rp = reinterpret_cast<const uint4*>(a.rows) + (live ? p : 0);
      const size_t gs = (size_t)a.ld;  // 16-byte words between groups of a row
      auto fetch = [&](int t0, uint4& d0, uint4& d1) {
        if (t0 < wmax) {
          d0 = __ldg(rp + (size_t)(t0 >> 3) * gs);
          d1 = __ldg(rp + (size_t)((t0 >> 3) + 1) * gs);
        } else {
          d0 = d1 = make_uint4(0u, 0u, 0u, 0u);
        }
      };
      uint4 n0, n1;
      fetch(0, n0, n1);
      for (int t0 = 0; t0 < wmax; t0 += kClusterTileSlots) {
        const uint32_t cu[8] = {n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, n1.z, n1.w};
        fetch(t0 + kClusterTileSlots, n0, n1);  // next chunk in flight
        // entries are byte offsets of the staged positions (16 q)
        auto get = [&](int kk) {
          return (int)((pick8(cu, kk >> 1) >> ((kk & 1) * 16)) & 0xFFF0u) >> 4;
        };
        if (!fast)
          chunk16(get, L - t0, wmax - t0);
        else if (live)
          chunk16_fast(get);
      }
    } else if (!tripped) {
      const int L = live ? (int)a.len[p] : 0;
      int wmax = L;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
      if ((tid & 31) == 0) s_max[tid >> 5] = wmax;
      __syncthreads();
      int maxl = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) maxl = max(maxl, s_max[w]);
      __syncthreads();  // s_max is rewritten by the next pass
      const int T = (maxl + kClusterTileSlots - 1) / kClusterTileSlots;
      const int x0 = base & ~7;  // 16-byte aligned start of the tile
      const int col = live ? p - x0 : tid;
      if (tid == 0) {
        for (int t = 0; t < nbuf && t < T; t++) {
          fence_proxy_async();
          mbar_expect_tx(&bar[t], tile_bytes);
          tma_load_2d(tiles + t * tile_elems, &rmap, x0, t * kClusterTileSlots, &bar[t]);
          inflight |= 1u << t;
        }
      }
      bool failed = false;
      int b = 0;  // buffer of tile t: t mod nbuf
      for (int t = 0; t < T; t++, b = b + 1 == nbuf ? 0 : b + 1) {
        const bool got = mbar_wait(&bar[b], (phase >> b) & 1u, a.status, a.wait_limit);
        const int wrem = wmax - t * kClusterTileSlots;  // warp-uniform
        if (got) {
          phase ^= 1u << b;
          inflight &= ~(1u << b);
          if (wrem > 0) {
            const uint16_t* tl = tiles + b * tile_elems + col;
            auto get = [&](int kk) { return (int)tl[kk * BX]; };
            if (!fast)
              chunk16(get, L - t * kClusterTileSlots, wrem);
            else if (live)
              chunk16_fast(get);
          }
        }
        // everyone is done with buffer b (and every wait succeeded)
        if (!__syncthreads_and(got)) {
          failed = true;
          break;
        }
        if (tid == 0 && t + nbuf < T) {
          fence_proxy_async();
          mbar_expect_tx(&bar[b], tile_bytes);
          tma_load_2d(tiles + b * tile_elems, &rmap, x0, (t + nbuf) * kClusterTileSlots, &bar[b]);
          inflight |= 1u << b;
        }
      }
      if (failed) {
        // a bounded wait ran out: give copies still in flight a bounded
        // chance to land in this block's shared memory, then leave
        if (tid == 0)
          for (int k = 0; k < nbuf; k++)
            if ((inflight >> k) & 1u) mbar_drain(&bar[k], (phase >> k) & 1u, a.status);
        aborted = true;
        break;
      }
    } else if (live) {
      // skin exceeded: the full candidate row from shared memory, and a
      // fresh compact row at the current positions
      int kept = 0, inchunk = 0;
      float cx = 0.f, cy = 0.f, cz = 0.f;
      walk_staged(sh, self, [&](int q) {
        pair(q, true, cx, cy, cz);
        if (++inchunk == kClusterTileSlots) {
          kahan_add(hx, lx, cx);
          kahan_add(hy, ly, cy);
          kahan_add(hz, lz, cz);
          fold_energy();
          cx = cy = cz = 0.f;
          inchunk = 0;
        }
        const float4 pj = st[q];
        float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        if (minimg) {
          dx = min_img(dx, Lf, invL);
          dy = min_img(dy, Lf, invL);
          dz = min_img(dz, Lf, invL);
        }
        if (dx * dx + dy * dy + dz * dz < a.rv2) {
          if (kept < a.cap) a.rows[row_slot(kept, p, a.ld, a.grouped)] = row_val(q, a.grouped);
          kept++;
        }
      });
      kahan_add(hx, lx, cx);
      kahan_add(hy, ly, cy);
      kahan_add(hz, lz, cz);
      fold_energy();
      if (kept > a.cap) atomicOr(&a.skin[3], 1);
      a.len[p] = (uint16_t)(kept < a.cap ? kept : a.cap);
      kept_new = kept;
      a.pos_build[p] = a.posf[p];
    }
    if (fast && !tripped && live && band_any) {
      LjParams lp;
      lp.s2[0] = s2_n, lp.s2[1] = s2_o, lp.s2[2] = s2_ng;
      lp.c24[0] = c_n, lp.c24[1] = c_o, lp.c24[2] = c_ng;
      lp.p = lj_p, lp.q = lj_q;
      const float3 e = band_pass<ALL_NG>(sh, st, a.pos, a.rcutsq, a.rows, a.ld, a.grouped, p,
                                         (int)a.len[p], pi, rc_lo, rc_hi, lp);
      kahan_add(hx, lx, e.x);
      kahan_add(hy, ly, e.y);
      kahan_add(hz, lz, e.z);
    }
    if (tripped) pad_rows_any(a.rows, a.ld, a.cap, p, live, kept_new, sh.S.staged, a.grouped);
    if (live) {
      // the compensated sums widened exactly (integer operations) and
      // combined in FP64
      const double f[3] = {widen_exact(hx) - widen_exact(lx), widen_exact(hy) - widen_exact(ly),
                           widen_exact(hz) - widen_exact(lz)};
      if (ENERGY) {
        ev[0] += (double)eh - (double)el;
        ev[1] += (double)sh2 - (double)sl2;
        ev[2] += 0.5 * ((double)wh - (double)wl);
      }
      if (GEAR != 1) {
        a.f3[3 * p] = f[0];
        a.f3[3 * p + 1] = f[1];
        a.f3[3 * p + 2] = f[2];
      }
      if (GEAR) {
        const md_double4 r = a.pos[p];
        const int type = ti;  // the staged copy carries the species as an integer
        GearAtom s;
        s.r[0] = r.x;
        s.r[1] = r.y;
        s.r[2] = r.z;
#pragma unroll
        for (int d = 0; d < 3; d++) {
          s.v[d] = a.g.vel[3 * p + d];
          s.a[d] = a.g.acc[3 * p + d];
          s.b[d] = a.g.b[3 * p + d];
          s.c[d] = a.g.c[3 * p + d];
        }
        const double im = type == SP_N ? a.g.inv_mass[0]
                                       : (type == SP_O ? a.g.inv_mass[1] : a.g.inv_mass[2]);
        gear_correct_fma(s, f, im, a.g.k);
        if (GEAR == 1) gear_predict_fma(s, a.g.k);
#pragma unroll
        for (int d = 0; d < 3; d++) {
          a.g.vel[3 * p + d] = s.v[d];
          a.g.acc[3 * p + d] = s.a[d];
          a.g.b[3 * p + d] = s.b[d];
          a.g.c[3 * p + d] = s.c[d];
        }
        md_double4 rn;
        rn.x = s.r[0];
        rn.y = s.r[1];
        rn.z = s.r[2];
        rn.w = r.w;
        a.g.pos_next[p] = rn;
        const float4 pf = make_float4(narrow_rn(s.r[0]), narrow_rn(s.r[1]), narrow_rn(s.r[2]),
                                      __int_as_float(type));
        // a non-finite force, velocity or derivative reaches the predicted
        // (corrected) position: one FP32 test covers the whole state
        if (!(fabsf(pf.x) <= FLT_MAX && fabsf(pf.y) <= FLT_MAX && fabsf(pf.z) <= FLT_MAX))
          atomicOr(a.status, ST_NONFINITE);
        a.g.posf_next[p] = pf;
        const float4 pb = a.pos_build[p];
        const float ddx = pf.x - pb.x, ddy = pf.y - pb.y, ddz = pf.z - pb.z;
        trip_next |= ddx * ddx + ddy * ddy + ddz * ddz > a.g.trip2;
      }
    }
  }
  if (aborted) break;
  if (ENERGY) block_sums_at<3>(ev, a.epart, sidx);
  __syncthreads();  // the next segment overwrites sh and the stage
  }
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&a.sched[1], 1) == (int)gridDim.x - 1) {
      a.sched[0] = 0;
      a.sched[1] = 0;
    }
  }
  if (GEAR && trip_next) a.skin[a.flag_set] = 1;
  if (blockIdx.x == 0 && tid == 0) {
    if (tripped) atomicAdd(&a.skin[4], 1);
    a.skin[a.flag_clear] = 0;  // flag of step t + 2 starts clear
  }
}

// ---- the lean kernel: one species, grouped rows, no energies ----
// The launches that run every step of the precision form (one species,
// grouped rows of the register-prefetch scheme, no energy terms) in a kernel
// of their own, with the same arithmetic as k_lj_cl<false, true, GEAR, 1>
// to the bit.  Only the padded-row pair loop and the Gear update are inline;
// the rare paths (the full-row walk of a skin trip, the minimum-image loop
// of one-cell replicas, the cutoff-band pass) are separate functions, so
// that their registers do not weigh on the pair loop.

struct LeanConst {
  float rc_lo, rc_hi, rc_mid, rc_half, lj_p, lj_q;
  float Lf, invL;
};

// F/r of one species, inv = 1/r^2: inv^4 (P inv^3 - Q) (k_lj_cl's lj_factor)
__device__ __forceinline__ float lean_factor(float r2, const LeanConst& k) {
  const float inv = rcp_approx(r2);
  const float inv2 = inv * inv;
  return (inv2 * inv2) * fmaf(k.lj_p, inv2 * inv, -k.lj_q);
}

struct LeanSum {
  float hx, hy, hz, lx, ly, lz;
  int kept;
};

// entry kk (0..15) of a 16-slot chunk held in two words of four
__device__ __forceinline__ int lean_entry(uint4 w0, uint4 w1, int kk) {
  const uint32_t c[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
  return (int)((pick8(c, kk >> 1) >> ((kk & 1) * 16)) & 0xFFF0u) >> 4;
}

// one checked pair of the walks below (k_lj_cl's pair, one species)
__device__ __forceinline__ void lean_checked(const SegShared& sh, const float4* st,
                                             const md_double4* pos, double rcutsq, int p,
                                             float4 pi, int q, bool valid, bool minimg,
                                             const LeanConst& k, float& cx, float& cy,
                                             float& cz) {
  const float4 pj = st[q];
  float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
  if (minimg) {
    dx = min_img(dx, k.Lf, k.invL);
    dy = min_img(dy, k.Lf, k.invL);
    dz = min_img(dz, k.Lf, k.invL);
  }
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  float fij = lean_factor(r2, k);
  bool in = r2 <= k.rc_lo;
  if (valid && !in && r2 < k.rc_hi) in = band_inside(sh, pos, p, q, rcutsq);
  in = in && valid;
  fij = in ? fij : 0.0f;
  cx = fmaf(dx, fij, cx);
  cy = fmaf(dy, fij, cy);
  cz = fmaf(dz, fij, cz);
}

// skin exceeded: the full candidate row from the stage, and a fresh compact
// row at the current positions (k_lj_cl's tripped path)
__device__ __noinline__ LeanSum lean_refresh(const SegShared& sh, const float4* st, const ClStep& a,
                                             int p, int self, float4 pi, LeanConst k) {
  LeanSum s = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};
  const bool minimg = sh.r.G == 1;
  int inchunk = 0;
  float cx = 0.f, cy = 0.f, cz = 0.f;
  walk_staged(sh, self, [&](int q) {
    lean_checked(sh, st, a.pos, a.rcutsq, p, pi, q, true, minimg, k, cx, cy, cz);
    if (++inchunk == kClusterTileSlots) {
      kahan_add(s.hx, s.lx, cx);
      kahan_add(s.hy, s.ly, cy);
      kahan_add(s.hz, s.lz, cz);
      cx = cy = cz = 0.f;
      inchunk = 0;
    }
    const float4 pj = st[q];
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    if (minimg) {
      dx = min_img(dx, k.Lf, k.invL);
      dy = min_img(dy, k.Lf, k.invL);
      dz = min_img(dz, k.Lf, k.invL);
    }
    if (dx * dx + dy * dy + dz * dz < a.rv2) {
      if (s.kept < a.cap) a.rows[row_slot(s.kept, p, a.ld, 1)] = row_val(q, 1);
      s.kept++;
    }
  });
  kahan_add(s.hx, s.lx, cx);
  kahan_add(s.hy, s.ly, cy);
  kahan_add(s.hz, s.lz, cz);
  if (s.kept > a.cap) atomicOr(&a.skin[3], 1);
  a.len[p] = (uint16_t)(s.kept < a.cap ? s.kept : a.cap);
  a.pos_build[p] = a.posf[p];
  return s;
}

// one-cell replicas (minimum images): the checked loop over the grouped
// row (k_lj_cl's chunk16), lanes of the warp in step; warp-collective
__device__ __noinline__ LeanSum lean_minimg(const SegShared& sh, const float4* st, const ClStep& a,
                                            int p, bool live, int self, float4 pi, LeanConst k) {
  LeanSum s = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};
  const int L = live ? (int)a.len[p] : 0;
  int wmax = L;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
  const uint4* rp = reinterpret_cast<const uint4*>(a.rows) + (live ? p : 0);
  for (int t0 = 0; t0 < wmax; t0 += kClusterTileSlots) {
    const uint4 w0 = __ldg(rp + (size_t)(t0 >> 3) * a.ld);
    const uint4 w1 = __ldg(rp + (size_t)((t0 >> 3) + 1) * a.ld);
    const int rem = L - t0, wrem = wmax - t0;
    float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
    for (int kk = 0; kk < kClusterTileSlots && kk < wrem; kk++) {
      const bool valid = kk < rem;
      const int q = valid ? lean_entry(w0, w1, kk) : self;
      if (kk & 1)
        lean_checked(sh, st, a.pos, a.rcutsq, p, pi, q, valid, true, k, bx, by, bz);
      else
        lean_checked(sh, st, a.pos, a.rcutsq, p, pi, q, valid, true, k, ax, ay, az);
    }
    kahan_add(s.hx, s.lx, ax + bx);
    kahan_add(s.hy, s.ly, ay + by);
    kahan_add(s.hz, s.lz, az + bz);
  }
  return s;
}

// 72 registers (7 blocks of 128 threads per SM): fewer spills than at 64
// registers and 8 blocks, which paid more than the eighth block did; blocks
// of up to 224 threads stay launchable for the autotuner.
template <int GEAR>
__global__ void __launch_bounds__(224, 4) k_lj_lean(const ClStep a) {
  extern __shared__ __align__(128) unsigned char dyn[];
  float4* st = reinterpret_cast<float4*>(dyn);
  const int tid = threadIdx.x;
  __shared__ SegShared sh;
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_trip, s_seg;
  if (tid == 0) {
    s_trip = (a.skin[a.flag_read] | a.skin[3]) != 0;
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool tripped = s_trip != 0;
  LeanConst k;
  k.rc_lo = a.lean_c[0];
  k.rc_hi = a.lean_c[1];
  k.rc_mid = a.lean_c[2];
  k.rc_half = a.lean_c[3];
  k.lj_p = a.lean_c[4];
  k.lj_q = a.lean_c[5];
  uint32_t phase = 0u;
  bool trip_next = false;
  for (;;) {
    if (tid == 0) s_seg = atomicAdd(&a.sched[0], 1);
    __syncthreads();
    const int sidx = s_seg;
    if (sidx >= a.nseg) break;
    load_segment(sh, a.seg, a.reps, sidx);
    __syncthreads();
    if (!stage_bulk(sh, a.posf, st, &bar, phase, a.status, a.wait_limit)) break;
    phase ^= 1u;
    put_sentinel(st, sh.S.staged);
    if (tripped) fill_offsets(sh, a.start);
    __syncthreads();
    const bool minimg = sh.r.G == 1;
    k.Lf = sh.r.Lf;
    k.invL = 1.0f / sh.r.Lf;
    const int p1 = sh.S.p1;
    for (int base = sh.S.p0; base < p1; base += blockDim.x) {
      const int p = base + tid;
      const bool live = p < p1;
      const int self = live ? self_offset(sh, p) : 0;
      if (GEAR && live) {
        prefetch_l2(a.pos + p);
        prefetch_l2(a.g.vel + 3 * (size_t)p);
        prefetch_l2(a.g.acc + 3 * (size_t)p);
        prefetch_l2(a.g.b + 3 * (size_t)p);
        prefetch_l2(a.g.c + 3 * (size_t)p);
        prefetch_l2(a.pos_build + p);
      }
      const float4 pi = st[self];
      float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
      if (tripped || minimg) {
        const LeanSum r = tripped ? (live ? lean_refresh(sh, st, a, p, self, pi, k) : LeanSum{})
                                  : lean_minimg(sh, st, a, p, live, self, pi, k);
        hx = r.hx, hy = r.hy, hz = r.hz, lx = r.lx, ly = r.ly, lz = r.lz;
        if (tripped) pad_rows_any(a.rows, a.ld, a.cap, p, live, r.kept, sh.S.staged, 1);
      } else {
        // the sentinel-padded rows: every slot below the warp's padded
        // length holds a real or a sentinel entry
        const int L = live ? (int)a.len[p] : 0;
        int wmax = L;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
        const uint4* rp = reinterpret_cast<const uint4*>(a.rows) + (live ? p : 0);
        const size_t gs = (size_t)a.ld;
        uint4 n0 = make_uint4(0u, 0u, 0u, 0u), n1 = n0;
        if (wmax > 0) {
          n0 = __ldg(rp);
          n1 = __ldg(rp + gs);
        }
        const char* sb = reinterpret_cast<const char*>(st);
        bool band_any = false;
        for (int t0 = 0; t0 < wmax; t0 += kClusterTileSlots) {
          const uint4 w0 = n0, w1 = n1;
          if (t0 + kClusterTileSlots < wmax) {
            n0 = __ldg(rp + (size_t)((t0 >> 3) + 2) * gs);
            n1 = __ldg(rp + (size_t)((t0 >> 3) + 3) * gs);
          }
          if (!live) continue;
          const uint32_t cw[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
          float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
          bool band = false;
          auto one = [&](uint32_t off, float& cx, float& cy, float& cz) {
            const float4 pj = *reinterpret_cast<const float4*>(sb + off);
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            float fij = lean_factor(r2, k);
            band |= fabsf(r2 - k.rc_mid) < k.rc_half;
            fij = r2 <= k.rc_lo ? fij : 0.0f;
            cx = fmaf(dx, fij, cx);
            cy = fmaf(dy, fij, cy);
            cz = fmaf(dz, fij, cz);
          };
#pragma unroll
          for (int w = 0; w < 8; w++) {
            one(cw[w] & 0xFFFFu, ax, ay, az);
            one(cw[w] >> 16, bx, by, bz);
          }
          band_any |= band;
          kahan_add(hx, lx, ax + bx);
          kahan_add(hy, ly, ay + by);
          kahan_add(hz, lz, az + bz);
        }
        if (live && band_any) {
          LjParams lp;
          lp.p = k.lj_p, lp.q = k.lj_q;
          const float3 e = band_pass<true>(sh, st, a.pos, a.rcutsq, a.rows, a.ld, 1, p, L, pi,
                                           k.rc_lo, k.rc_hi, lp);
          kahan_add(hx, lx, e.x);
          kahan_add(hy, ly, e.y);
          kahan_add(hz, lz, e.z);
        }
      }
      if (!live) continue;
      const double f[3] = {widen_exact(hx) - widen_exact(lx), widen_exact(hy) - widen_exact(ly),
                           widen_exact(hz) - widen_exact(lz)};
      if (GEAR != 1) {
        a.f3[3 * p] = f[0];
        a.f3[3 * p + 1] = f[1];
        a.f3[3 * p + 2] = f[2];
      }
      if (GEAR) {
        const md_double4 r = a.pos[p];
        const int type = __float_as_int(pi.w);
        GearAtom s;
        s.r[0] = r.x;
        s.r[1] = r.y;
        s.r[2] = r.z;
#pragma unroll
        for (int d = 0; d < 3; d++) {
          s.v[d] = a.g.vel[3 * p + d];
          s.a[d] = a.g.acc[3 * p + d];
          s.b[d] = a.g.b[3 * p + d];
          s.c[d] = a.g.c[3 * p + d];
        }
        const double im = type == SP_N ? a.g.inv_mass[0]
                                       : (type == SP_O ? a.g.inv_mass[1] : a.g.inv_mass[2]);
        gear_correct_fma(s, f, im, a.g.k);
        if (GEAR == 1) gear_predict_fma(s, a.g.k);
#pragma unroll
        for (int d = 0; d < 3; d++) {
          a.g.vel[3 * p + d] = s.v[d];
          a.g.acc[3 * p + d] = s.a[d];
          a.g.b[3 * p + d] = s.b[d];
          a.g.c[3 * p + d] = s.c[d];
        }
        md_double4 rn;
        rn.x = s.r[0];
        rn.y = s.r[1];
        rn.z = s.r[2];
        rn.w = r.w;
        a.g.pos_next[p] = rn;
        const float4 pf = make_float4(narrow_rn(s.r[0]), narrow_rn(s.r[1]), narrow_rn(s.r[2]),
                                      __int_as_float(type));
        if (!(fabsf(pf.x) <= FLT_MAX && fabsf(pf.y) <= FLT_MAX && fabsf(pf.z) <= FLT_MAX))
          atomicOr(a.status, ST_NONFINITE);
        a.g.posf_next[p] = pf;
        const float4 pb = a.pos_build[p];
        const float ddx = pf.x - pb.x, ddy = pf.y - pb.y, ddz = pf.z - pb.z;
        trip_next |= ddx * ddx + ddy * ddy + ddz * ddz > a.g.trip2;
      }
    }
    __syncthreads();  // the next segment overwrites sh and the stage
  }
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&a.sched[1], 1) == (int)gridDim.x - 1) {
      a.sched[0] = 0;
      a.sched[1] = 0;
    }
  }
  if (GEAR && trip_next) a.skin[a.flag_set] = 1;
  if (blockIdx.x == 0 && tid == 0) {
    if (tripped) atomicAdd(&a.skin[4], 1);
    a.skin[a.flag_clear] = 0;
  }
}

// reference-layout rows, original numbering (single replica)
__global__ void __launch_bounds__(256)
    k_cl_ref_rows(const ClusterSegment* __restrict__ seg, const ClusterReplica* __restrict__ reps,
                  const int* __restrict__ start, const int* __restrict__ orig,
                  const md_double4* __restrict__ pos, int nls, int* __restrict__ out,
                  signed char* __restrict__ img, int* __restrict__ nlargest) {
  __shared__ SegShared sh;
  load_segment(sh, seg, reps, blockIdx.x);
  __syncthreads();
  fill_offsets(sh, start);
  __syncthreads();
  const double L = sh.r.L;
  for (int p = sh.S.p0 + threadIdx.x; p < sh.S.p1; p += blockDim.x) {
    const int self = self_offset(sh, p);
    const size_t o = (size_t)orig[p] * nls;
    const md_double4 a = pos[p];
    int k = 0;
    walk_staged(sh, self, [&](int q) {
      int ix, iy, iz;
      const int j = staged_source(sh.S, q, ix, iy, iz);
      if (sh.r.G == 1) {
        const md_double4 b = pos[j];
        ix = min_image(a.x, b.x, L);
        iy = min_image(a.y, b.y, L);
        iz = min_image(a.z, b.z, L);
      }
      if (out && k < nls) {
        out[o + k] = orig[j];
        if (img) img[o + k] = (signed char)((ix + 1) * 9 + (iy + 1) * 3 + (iz + 1));
      }
      k++;
    });
    atomicMax(nlargest, k);
    if (!out) continue;
    for (; k < nls; k++) {
      out[o + k] = -1;
      if (img) img[o + k] = 13;
    }
  }
}

__global__ void k_unpermute(const double* __restrict__ in, double* __restrict__ out,
                            const int* __restrict__ orig, int n, int width) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const size_t o = (size_t)orig[p];
  for (int d = 0; d < width; d++) out[width * o + d] = in[(size_t)width * p + d];
}

__global__ void k_invert(const int* __restrict__ orig, int* __restrict__ inv, int n) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) inv[orig[p]] = p;
}

// one element per thread in the caller's order: the host side is read or
// written in whole consecutive lines (W is 3 or 4; W n < 2^31)
template <int W>
__global__ void k_gather_host(const double* __restrict__ host, double* __restrict__ dst,
                              const int* __restrict__ inv, int m) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const int i = k / W;
    dst[(size_t)W * inv[i] + (k - i * W)] = host[k];
  }
}

template <int W>
__global__ void k_scatter_host(const double* __restrict__ src, double* __restrict__ host,
                               const int* __restrict__ inv, int m) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const int i = k / W;
    host[k] = src[(size_t)W * inv[i] + (k - i * W)];
  }
}

__global__ void k_species_check(const md_double4* __restrict__ pos, int n, int* flag) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool other = p < n && (int)pos[p].w != SP_NG;
  if (__any_sync(0xffffffffu, other) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

__global__ void k_permute_in(const double* __restrict__ in, double* __restrict__ out,
                             const int* __restrict__ orig, int n, int width) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const size_t o = (size_t)orig[p];
  for (int d = 0; d < width; d++) out[(size_t)width * p + d] = in[width * o + d];
}

__global__ void k_iota(int* __restrict__ a, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = i;
}

inline int nb(long long n, int t) { return (int)((n + t - 1) / t); }

template <typename T>
cudaError_t realloc_dev(T*& p, size_t count) {
  if (p) cudaFree(p);
  p = nullptr;
  return cudaMalloc(&p, sizeof(T) * (count > 0 ? count : 1));
}

// staged positions plus the far sentinel that pads the rows (entry `staged`)
size_t stage_bytes(int staged) { return sizeof(float4) * ((size_t)std::max(staged, 1) + 1); }

template <typename K>
void allow_smem(K kern) {
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(float4) * (kClusterMaxStaged + 1) +
                             std::max(3 * kClusterTileSlots * 256 * sizeof(uint16_t),
                                      (size_t)8 * 2 * kWarpTileBytes)));
}

}  // namespace

int cluster_blocks(const ClusterList& cl) { return cl.nseg; }

int cluster_build(ClusterList& cl, const std::vector<ClusterReplica>& reps_in, float rv,
                  double rcut, md_double4** pos, double** v3[5], float4* posf, Scratch& sc,
                  int* d_status, cudaStream_t st, std::string& err) {
  cudaError_t e;
  if (cl.block < 32 || cl.block > 248 || cl.block % 32) {
    err = "cluster block size must be a multiple of 32 up to 224";
    return -1;
  }
  // replica geometry (host): cells and columns
  std::vector<ClusterReplica> reps = reps_in;
  int natoms = 0, cell0 = 0, col0 = 0;
  for (auto& r : reps) {
    if (!(r.L > 2.0 * (double)rv)) {
      err = "periodic box must exceed twice the list radius";
      return -1;
    }
    r.atom0 = natoms;
    natoms += r.n;
    int G = (int)floor(r.L / (double)rv);
    if (G < 3) G = 1;
    r.G = G;
    r.pad = 0;
    r.cs = r.L / G;
    r.invL = 1.0 / r.L;
    r.invcs = 1.0 / r.cs;
    r.Lf = (float)r.L;
    r.Llo = (float)(r.L - (double)r.Lf);
    r.cell0 = cell0;
    r.col0 = col0;
    cell0 += G == 1 ? 1 : G * G * G;
    col0 += G == 1 ? 1 : G * G;
  }
  if (natoms > kMaxAtoms) {
    err = "too many atoms";
    return -1;
  }
  const int n = natoms;
  const bool new_geometry = cl.h_rep.size() != reps.size() || !cl.rep ||
                            memcmp(cl.h_rep.data(), reps.data(),
                                   sizeof(ClusterReplica) * reps.size()) != 0;
  cl.nrep = (int)reps.size();
  cl.natoms = n;
  cl.h_rep = reps;
  cl.ncells = cell0;
  cl.ncols = col0;
  if (new_geometry) {
    if ((e = realloc_dev(cl.rep, reps.size())) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(cl.rep, reps.data(), sizeof(ClusterReplica) * reps.size(),
                             cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return e;
    // the copy reads cl.h_rep, which stays alive; no wait needed
  }
  if (cl.ncells + 1 > cl.cells_alloc) {
    for (int** p : {&cl.count, &cl.start, &cl.fill, &cl.segidx})
      if ((e = realloc_dev(*p, (size_t)cl.ncells + 1)) != cudaSuccess) return e;
    if ((e = realloc_dev(cl.seg, (size_t)cl.ncells)) != cudaSuccess) return e;
    cl.cells_alloc = cl.ncells + 1;
    cl.seg_alloc = cl.ncells;
  }
  if (n > cl.n_alloc) {
    for (int** p : {&cl.cell, &cl.unsorted, &cl.perm, &cl.itmp})
      if ((e = realloc_dev(*p, (size_t)n)) != cudaSuccess) return e;
    if ((e = realloc_dev(cl.orig, (size_t)n)) != cudaSuccess) return e;
    k_iota<<<nb(n, 256), 256, 0, st>>>(cl.orig, n);  // first build: identity
    if ((e = realloc_dev(cl.len, (size_t)n)) != cudaSuccess) return e;
    if ((e = realloc_dev(cl.pos_build, (size_t)n)) != cudaSuccess) return e;
    if ((e = realloc_dev(cl.pos_tmp, (size_t)n)) != cudaSuccess) return e;
    for (int k = 0; k < 5; k++)
      if (v3[k] && *v3[k] && (e = realloc_dev(cl.v3_tmp[k], 3 * (size_t)n)) != cudaSuccess)
        return e;
    cl.n_alloc = n;
  }
  if (!cl.skin) {
    if ((e = cudaMalloc(&cl.skin, sizeof(int) * 8)) != cudaSuccess) return e;
    cudaMemsetAsync(cl.skin, 0, sizeof(int) * 8, st);
  }
  if (!cl.counters && (e = cudaMalloc(&cl.counters, sizeof(int) * 8)) != cudaSuccess) return e;
  if (!cl.sched) {
    if ((e = cudaMalloc(&cl.sched, sizeof(int) * 2)) != cudaSuccess) return e;
    cudaMemsetAsync(cl.sched, 0, sizeof(int) * 2, st);
  }
  cudaMemsetAsync(cl.counters, 0, sizeof(int) * 8, st);
  cudaMemsetAsync(cl.count, 0, sizeof(int) * ((size_t)cl.ncells + 1), st);
  cudaMemsetAsync(cl.fill, 0, sizeof(int) * ((size_t)cl.ncells + 1), st);
  const int T = 256;
  if (n > 0)
    k_cl_assign<<<nb(n, T), T, 0, st>>>(*pos, n, cl.rep, cl.nrep, cl.cell, cl.count, cl.counters,
                                        d_status);
  if ((e = scan_exclusive(cl.count, cl.start, cl.ncells + 1, sc, st)) != cudaSuccess) return e;
  if (n > 0) {
    k_cl_scatter<<<nb(n, T), T, 0, st>>>(cl.cell, n, cl.start, cl.fill, cl.unsorted);
    k_cl_rank<<<nb(n, T), T, 0, st>>>(cl.unsorted, cl.cell, cl.orig, n, cl.start, cl.perm);
    // permute the state into cell order
    k_gather<md_double4><<<nb(n, T), T, 0, st>>>(*pos, cl.pos_tmp, cl.perm, n);
    std::swap(*pos, cl.pos_tmp);
    for (int k = 0; k < 5; k++)
      if (v3[k] && *v3[k]) {
        k_gather3<<<nb(n, T), T, 0, st>>>(*v3[k], cl.v3_tmp[k], cl.perm, n);
        std::swap(*v3[k], cl.v3_tmp[k]);
      }
    k_gather<int><<<nb(n, T), T, 0, st>>>(cl.orig, cl.itmp, cl.perm, n);
    std::swap(cl.orig, cl.itmp);
    k_cl_posf<<<nb(n, T), T, 0, st>>>(*pos, cl.pos_build, posf, n);
  }
  // segments: greedy cut of the columns (fill is free again and holds the flags)
  const int zmax = std::max(1, std::min(cl.Z, kClusterMaxZ));
  k_seg_flags<<<nb(cl.ncols, 128), 128, 0, st>>>(cl.rep, cl.nrep, cl.ncols, cl.ncells, cl.count,
                                                 cl.fill, cl.block,
                                                 std::min(cl.stage_cap, kClusterMaxStaged), zmax);
  if ((e = scan_exclusive(cl.fill, cl.segidx, cl.ncells + 1, sc, st)) != cudaSuccess) return e;
  k_seg_emit<<<nb(cl.ncells, 256), 256, 0, st>>>(cl.rep, cl.nrep, cl.ncells, cl.fill, cl.segidx,
                                                 cl.seg);
  k_cl_segments<<<nb(cl.ncells, 128), 128, 0, st>>>(cl.seg, cl.segidx + cl.ncells, cl.rep,
                                                    cl.start, cl.counters);
  int hc[8];
  int status = 0, nseg = 0;
  cudaMemcpyAsync(hc, cl.counters, sizeof(hc), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&nseg, cl.segidx + cl.ncells, sizeof(int), cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  if (status & ST_NONFINITE) {
    err = "non-finite position at list build";
    return -1;
  }
  cl.nseg = nseg;
  cl.max_staged = hc[0];
  cl.maxcell = hc[4];
  if (cl.max_staged > kClusterMaxStaged) {
    err = "segment neighbourhood of " + std::to_string(cl.max_staged) +
          " atoms exceeds the shared-memory stage (use fewer cells per segment)";
    return -1;
  }
  static bool attrs = false;
  if (!attrs) {
    allow_smem(k_cl_rows<0>);
    allow_smem(k_cl_rows<1>);
    allow_smem(k_cl_rows<2>);
    allow_smem(k_lj_cl<false, false, 0, 0>);
    allow_smem(k_lj_cl<false, true, 0, 0>);
    allow_smem(k_lj_cl<true, false, 0, 0>);
    allow_smem(k_lj_cl<true, true, 0, 0>);
    allow_smem(k_lj_cl<false, false, 1, 0>);
    allow_smem(k_lj_cl<false, true, 1, 0>);
    allow_smem(k_lj_cl<false, false, 2, 0>);
    allow_smem(k_lj_cl<false, true, 2, 0>);
    allow_smem(k_lj_cl<false, false, 0, 1>);
    allow_smem(k_lj_cl<false, true, 0, 1>);
    allow_smem(k_lj_cl<true, false, 0, 1>);
    allow_smem(k_lj_cl<true, true, 0, 1>);
    allow_smem(k_lj_cl<false, false, 1, 1>);
    allow_smem(k_lj_cl<false, true, 1, 1>);
    allow_smem(k_lj_cl<false, false, 2, 1>);
    allow_smem(k_lj_cl<false, true, 2, 1>);
    allow_smem(k_lj_cl<false, false, 0, 2>);
    allow_smem(k_lj_cl<false, true, 0, 2>);
    allow_smem(k_lj_cl<true, false, 0, 2>);
    allow_smem(k_lj_cl<true, true, 0, 2>);
    allow_smem(k_lj_cl<false, false, 1, 2>);
    allow_smem(k_lj_cl<false, true, 1, 2>);
    allow_smem(k_lj_cl<false, false, 2, 2>);
    allow_smem(k_lj_cl<false, true, 2, 2>);
    allow_smem(k_lj_lean<0>);
    allow_smem(k_lj_lean<1>);
    allow_smem(k_lj_lean<2>);
    attrs = true;
  }
  // the register-prefetch scheme reads grouped rows of byte offsets, which
  // address at most 4,094 staged atoms and the sentinel; denser
  // neighbourhoods take the block-tile scheme
  if (cl.row_loads == 2 && cl.max_staged >= 4095) cl.row_loads = 1;
  const int grouped = cl.row_loads == 2 ? 1 : 0;
  if (grouped != cl.grouped) {
    cl.grouped = grouped;
    cl.cap = 0;  // the old rows are in the other layout: rebuild them
  }
  const float margin = (float)(1e-6 * (reps.empty() ? 0.0 : reps.back().L + rv) + 1e-6);
  const float rv_keep = rv + margin;
  cl.rv = rv;
  cl.rv2 = rv_keep * rv_keep;
  cl.ld = (std::max(n, 1) + 31) / 32 * 32;
  const size_t smem = stage_bytes(cl.max_staged);
  // one pass into the rows of the previous capacity when there are some;
  // a second (writing) pass only when a row outgrew them
  const bool have_rows = cl.rows && cl.cap > 0 && (long long)cl.cap * cl.ld <= cl.rows_elems;
  if (cl.nseg > 0) {
    if (have_rows)
      k_cl_rows<2><<<cl.nseg, cl.block, smem, st>>>(cl.seg, cl.rep, cl.start, cl.pos_build, cl.rv2,
                                               cl.rows, cl.len, cl.ld, cl.cap, cl.counters,
                                               cl.grouped);
    else
      k_cl_rows<0><<<cl.nseg, cl.block, smem, st>>>(cl.seg, cl.rep, cl.start, cl.pos_build, cl.rv2,
                                               nullptr, cl.len, cl.ld, 0, cl.counters, 0);
  }
  cudaMemcpyAsync(hc, cl.counters, sizeof(hc), cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  cl.maxlen = hc[1];
  {
    unsigned long long ent;
    memcpy(&ent, hc + 2, sizeof(ent));
    cl.entries = (long long)ent;
  }
  // whole 16-slot tiles: rows are padded to the warp's longest row rounded up
  const int want =
      std::min(65520, ((int)(std::max(cl.maxlen, 1) * cl.headroom) + 8 + kClusterTileSlots - 1) /
                          kClusterTileSlots * kClusterTileSlots);
  const bool fits = have_rows && want <= cl.cap;
  if (!fits) {
    cl.cap = want;
    const long long need = (long long)cl.cap * cl.ld;
    if (need > cl.rows_elems || !cl.rows) {
      if ((e = realloc_dev(cl.rows, (size_t)need)) != cudaSuccess) return e;
      cl.rows_elems = need;
    }
  }
  cl.rmap_ok = encode_tiled_2d(&cl.rmap, CU_TENSOR_MAP_DATA_TYPE_UINT16, cl.rows,
                               (uint64_t)cl.ld, (uint64_t)cl.cap, (uint64_t)cl.ld * 2,
                               (uint32_t)(cl.block + 8), (uint32_t)kClusterTileSlots) &&
               encode_tiled_2d(&cl.rmap_w, CU_TENSOR_MAP_DATA_TYPE_UINT16, cl.rows,
                               (uint64_t)cl.ld, (uint64_t)cl.cap, (uint64_t)cl.ld * 2,
                               (uint32_t)kWarpTileAtoms, (uint32_t)kClusterTileSlots);
  if (!cl.rmap_ok) {
    err = "TMA descriptor of the cluster rows could not be encoded";
    return -1;
  }
  if (!fits && cl.nseg > 0)
    k_cl_rows<1><<<cl.nseg, cl.block, smem, st>>>(cl.seg, cl.rep, cl.start, cl.pos_build, cl.rv2,
                                             cl.rows, cl.len, cl.ld, cl.cap, cl.counters,
                                             cl.grouped);
  cl.trip_dist = 0.5 * ((double)rv - rcut) - (double)margin;
  cudaMemsetAsync(cl.skin, 0, sizeof(int) * 4, st);  // trip flags and overflow
  cl.built = true;
  cl.version++;
  return (int)cudaGetLastError();
}

int cluster_occupancy_cap(int threads, int row_loads, bool all_ng) {
  // the kernel and row-tile bytes the fused every-step launch below uses
  const bool block_tiles = row_loads == 1 || row_loads == 4;
  const size_t tiles =
      block_tiles ? (row_loads == 4 ? 3 : 2) * kClusterTileSlots * (size_t)(threads + 8) *
                        sizeof(uint16_t)
                  : (row_loads == 3 ? (size_t)(threads / 32) * 2 * kWarpTileBytes : 0);
  const void* kern;
  if (row_loads == 2 && all_ng)
    kern = (const void*)k_lj_lean<1>;
  else if (block_tiles)
    kern = all_ng ? (const void*)k_lj_cl<false, true, 1, 0> : (const void*)k_lj_cl<false, false, 1, 0>;
  else if (row_loads == 3)
    kern = all_ng ? (const void*)k_lj_cl<false, true, 1, 2> : (const void*)k_lj_cl<false, false, 1, 2>;
  else
    kern = all_ng ? (const void*)k_lj_cl<false, true, 1, 1> : (const void*)k_lj_cl<false, false, 1, 1>;
  auto blocks = [&](int staged) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads,
                                                      tiles + stage_bytes(staged)) != cudaSuccess)
      nb = 0;
    return nb;
  };
  const int nb0 = blocks(1);
  if (nb0 < 1) return kClusterMaxStaged;
  int lo = 1, hi = kClusterMaxStaged;  // the largest stage with nb0 blocks per SM
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (blocks(mid) >= nb0) lo = mid; else hi = mid - 1;
  }
  return lo;
}

void launch_lj_cluster(const ClusterForceArgs& f, bool energy, cudaStream_t st) {
  const ClusterList& cl = *f.cl;
  if (cl.nseg == 0) return;
  const bool block_tiles = cl.row_loads == 1 || cl.row_loads == 4;
  const int nbuf = cl.row_loads == 4 ? 3 : 2;
  const size_t tiles =
      block_tiles ? nbuf * kClusterTileSlots * (size_t)(cl.block + 8) * sizeof(uint16_t)
                  : (cl.row_loads == 3 ? (size_t)(cl.block / 32) * 2 * kWarpTileBytes : 0);
  const size_t smem = tiles + stage_bytes(cl.max_staged);
  ClStep a;
  a.nseg = cl.nseg;
  a.sched = cl.sched;
  a.seg = cl.seg;
  a.reps = cl.rep;
  a.start = cl.start;
  a.posf = f.posf;
  a.pos = f.pos;
  a.f3 = f.f3;
  a.rows = cl.rows;
  a.len = cl.len;
  a.ld = cl.ld;
  a.cap = cl.cap;
  a.rv2 = cl.rv2;
  a.pos_build = cl.pos_build;
  a.skin = f.skin ? f.skin : cl.skin;
  a.flag_read = f.step % 3;
  a.flag_set = (f.step + 1) % 3;
  a.flag_clear = (f.step + 2) % 3;
  a.rcutsq = f.rcutsq;
  a.sp = f.sp;
  a.epart = f.epart;
  a.status = f.status;
  if (f.gear) a.g = *f.gear;
  else memset(&a.g, 0, sizeof(a.g));
  {
    const float rc2 = (float)f.rcutsq;
    const float lo = rc2 * (1.0f - 1e-5f), hi = rc2 * (1.0f + 1e-5f);
    const float s2 = f.sp.sig[2] * f.sp.sig[2], c24 = 24.0f * f.sp.eps[2];
    const float q6 = s2 * s2 * s2;
    a.lean_c[0] = lo;
    a.lean_c[1] = hi;
    a.lean_c[2] = 0.5f * (lo + hi);
    a.lean_c[3] = 0.5f * (hi - lo) * 1.001f;
    a.lean_c[4] = 2.0f * c24 * q6 * q6;
    a.lean_c[5] = c24 * q6;
  }
  a.nbuf = nbuf;
  a.wait_limit = f.wait_limit;
  a.grouped = cl.grouped;
  // persistent grid: as many blocks as fit on the GPU at once, at most one
  // per segment
  auto grid_for = [&](const void* kern) {
    static int sms = 0;
    if (!sms) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (sms <= 0) sms = 1;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, cl.block, smem) !=
            cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    return std::min(cl.nseg, sms * per_sm);
  };
#define MDGB_CL_LAUNCH2(E, A, G, T, M)                                                      \
  k_lj_cl<E, A, G, T><<<grid_for((const void*)k_lj_cl<E, A, G, T>), cl.block, smem, st>>>( \
      M, a)
#define MDGB_CL_LAUNCH(E, A, G)                  \
  if (block_tiles)                               \
    MDGB_CL_LAUNCH2(E, A, G, 0, cl.rmap);        \
  else if (cl.row_loads == 3)                    \
    MDGB_CL_LAUNCH2(E, A, G, 2, cl.rmap_w);      \
  else                                           \
    MDGB_CL_LAUNCH2(E, A, G, 1, cl.rmap)
  if (cl.grouped && f.all_ng && !energy) {
    // every-step launches of one species on grouped rows: the lean kernel
    const int gear = !f.gear ? 0 : (f.gear->correct_only ? 2 : 1);
    const size_t sm = stage_bytes(cl.max_staged);
    if (gear == 1)
      k_lj_lean<1><<<grid_for((const void*)k_lj_lean<1>), cl.block, sm, st>>>(a);
    else if (gear == 2)
      k_lj_lean<2><<<grid_for((const void*)k_lj_lean<2>), cl.block, sm, st>>>(a);
    else
      k_lj_lean<0><<<grid_for((const void*)k_lj_lean<0>), cl.block, sm, st>>>(a);
  } else if (energy) {
    if (f.all_ng) { MDGB_CL_LAUNCH(true, true, 0); } else { MDGB_CL_LAUNCH(true, false, 0); }
  } else if (f.gear && f.gear->correct_only) {
    if (f.all_ng) { MDGB_CL_LAUNCH(false, true, 2); } else { MDGB_CL_LAUNCH(false, false, 2); }
  } else if (f.gear) {
    if (f.all_ng) { MDGB_CL_LAUNCH(false, true, 1); } else { MDGB_CL_LAUNCH(false, false, 1); }
  } else {
    if (f.all_ng) { MDGB_CL_LAUNCH(false, true, 0); } else { MDGB_CL_LAUNCH(false, false, 0); }
  }
#undef MDGB_CL_LAUNCH
#undef MDGB_CL_LAUNCH2
}

int cluster_reference_rows(const ClusterList& cl, const md_double4* pos, int nlistsize,
                           int* d_out, signed char* d_img, int* d_nlargest, cudaStream_t st) {
  if (cl.nseg == 0) return 0;
  k_cl_ref_rows<<<cl.nseg, 128, 0, st>>>(cl.seg, cl.rep, cl.start, cl.orig, pos, nlistsize,
                                         d_out, d_img, d_nlargest);
  return (int)cudaGetLastError();
}

// per-replica sums of the per-segment LJ energies (segments of a replica
// are the contiguous range starting at the segment of its first cell)
__global__ void k_rep_energy(const ClusterReplica* __restrict__ reps, int nrep, int ncells,
                             const int* __restrict__ segidx, const double* __restrict__ epart,
                             double* __restrict__ out3) {
  const int k = blockIdx.x;
  const int s0 = segidx[reps[k].cell0];
  const int s1 = segidx[k + 1 < nrep ? reps[k + 1].cell0 : ncells];
  __shared__ double sm[3][32];
  double v[3] = {0.0, 0.0, 0.0};
  for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x)
    for (int d = 0; d < 3; d++) v[d] += epart[3 * (size_t)s + d];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = 0; d < 3; d++) {
    double x = v[d];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sm[d][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[threadIdx.x][w];
    out3[3 * k + threadIdx.x] = t;
  }
}

void launch_rep_energy(const ClusterList& cl, const double* epart, double* out3,
                       cudaStream_t st) {
  if (cl.nrep > 0)
    k_rep_energy<<<cl.nrep, 128, 0, st>>>(cl.rep, cl.nrep, cl.ncells, cl.segidx, epart, out3);
}

void launch_unpermute(const double* in, double* out, const int* orig, int n, int width,
                      cudaStream_t st) {
  if (n > 0) k_unpermute<<<nb(n, 256), 256, 0, st>>>(in, out, orig, n, width);
}

void launch_permute_in(const double* in, double* out, const int* orig, int n, int width,
                       cudaStream_t st) {
  if (n > 0) k_permute_in<<<nb(n, 256), 256, 0, st>>>(in, out, orig, n, width);
}

void launch_invert(const int* orig, int* inv, int n, cudaStream_t st) {
  if (n > 0) k_invert<<<nb(n, 256), 256, 0, st>>>(orig, inv, n);
}

void launch_gather_host(const double* host, double* dst, const int* inv, int n, int width,
                        cudaStream_t st) {
  const int m = n * width;
  if (m <= 0) return;
  const int g = std::min(nb(m, 256), 16 * 1024);
  if (width == 4)
    k_gather_host<4><<<g, 256, 0, st>>>(host, dst, inv, m);
  else
    k_gather_host<3><<<g, 256, 0, st>>>(host, dst, inv, m);
}

void launch_scatter_host(const double* src, double* host, const int* inv, int n, int width,
                         cudaStream_t st) {
  const int m = n * width;
  if (m <= 0) return;
  const int g = std::min(nb(m, 256), 16 * 1024);
  if (width == 4)
    k_scatter_host<4><<<g, 256, 0, st>>>(src, host, inv, m);
  else
    k_scatter_host<3><<<g, 256, 0, st>>>(src, host, inv, m);
}

void launch_species_check(const md_double4* pos, int n, int* flag, cudaStream_t st) {
  if (n > 0) k_species_check<<<nb(n, 256), 256, 0, st>>>(pos, n, flag);
}

void cluster_free(ClusterList& cl) {
  std::vector<void*> ptrs = {cl.rep,  cl.seg,      cl.count,     cl.start,   cl.fill, cl.segidx,
                             cl.cell, cl.unsorted, cl.perm,      cl.orig,    cl.itmp,
                             cl.rows, cl.len,      cl.pos_build, cl.pos_tmp, cl.skin,
                             cl.counters, cl.sched};
  for (int k = 0; k < 5; k++) ptrs.push_back(cl.v3_tmp[k]);
  for (void* p : ptrs)
    if (p) cudaFree(p);
  cl = ClusterList();
}

}  // namespace mdgb
