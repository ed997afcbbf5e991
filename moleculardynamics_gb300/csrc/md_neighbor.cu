// Neighbour-list build on the GPU (replaces common/NeighborList.cpp:14-207).
//
// Pipeline for atoms [0, n):
//   1. cell of every atom from its FP64 position with the reference's own
//      arithmetic, (int)((x + npos) / cellSize) (NeighborList.cpp:81-83), and
//      an open-addressing table of occupied cells (atomicCAS on 64-bit keys);
//   2. exclusive scan of the per-cell counts;
//   3. atoms scattered by cell, then ranked inside their cell so that each
//      cell lists its atoms in ascending index (NeighborList.cpp:104-117);
//   4. rows: the 27-cell stencil in the order dx, dy, dz = -1..1 with the
//      reference's bounds test (NeighborList.cpp:142-168).  Rows are counted
//      first, then written in ELL slot-major layout list[k * n + i].
// A compact list keeps, in row order, only the candidates within rv of the
// atom at build time; the step engine checks every step that no atom moved
// far enough for a dropped candidate to come within rcut, and otherwise walks
// the full row (same candidates, same order as the reference).
#include <cmath>
#include <cstdio>
#include <cstring>

#include "md_neighbor.cuh"

namespace mdgb {

namespace {

constexpr int kMaxCellCoord = (1 << 21) - 3;

__global__ void k_cell_assign(md_double4* __restrict__ pos, int n, Grid g, int* __restrict__ cell3,
                              unsigned long long* __restrict__ keys, int* __restrict__ count,
                              int cap, int* __restrict__ atom_slot, int* __restrict__ counters,
                              int* __restrict__ status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  md_double4 p = pos[i];
  double x[3] = {p.x, p.y, p.z};
  if (g.periodic) {
    // periodic extension: x - L * floor((x + L/2) / L)
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double q = floor(xdiv(xadd(x[d], g.npos), g.box));
      x[d] = xsub(x[d], xmul(q, g.box));
    }
    p.x = x[0];
    p.y = x[1];
    p.z = x[2];
    pos[i] = p;
  }
  int c[3];
  bool bad = false;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double q = xdiv(xadd(x[d], g.npos), g.cs);
    if (!(q >= 0.0 && q < (double)kMaxCellCoord)) {
      bad = true;
      q = 0.0;
    }
    c[d] = __double2int_rz(q);
    if (g.periodic) {
      if (c[d] >= g.cells) c[d] = g.cells - 1;
      if (c[d] < 0) c[d] = 0;
    }
  }
  // one 16-byte row per atom: x, y, z and an unused fourth int
  reinterpret_cast<int4*>(cell3)[i] = make_int4(c[0], c[1], c[2], 0);
  if (bad) atomicOr(status, isfinite(p.x + p.y + p.z) ? ST_CELL_OVERFLOW : ST_NONFINITE);
  unsigned long long key = cell_key(c[0], c[1], c[2]);
  unsigned h = (unsigned)(mix64(key) & (unsigned long long)(cap - 1));
  int probe = 0;
  for (; probe < cap; probe++) {
    unsigned long long prev = atomicCAS(&keys[h], kEmptyKey, key);
    if (prev == kEmptyKey || prev == key) break;
    h = (h + 1) & (unsigned)(cap - 1);
  }
  if (probe == cap) {
    atomicOr(status, ST_CELL_OVERFLOW);
    atom_slot[i] = 0;
    return;
  }
  atom_slot[i] = (int)h;
  int old = atomicAdd(&count[h], 1);
  const unsigned m = __activemask();
  const unsigned big = __reduce_max_sync(m, (unsigned)(old + 1));
  if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicMax(&counters[0], (int)big);
}

// exclusive scan, 4 items per thread, 1024 threads per block
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* smem, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int s = lane < (blockDim.x >> 5) ? smem[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    smem[lane] = s;
  }
  __syncthreads();
  int warp_prefix = warp > 0 ? smem[warp - 1] : 0;
  total = smem[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void k_scan_tiles(const int* __restrict__ in, int* __restrict__ out, int n,
                             int* __restrict__ tile_sums) {
  __shared__ int smem[32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int total;
  int pre = block_exclusive_scan(s, smem, total);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) out[base + k] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0 && tile_sums) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ tile_pre) {
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  const int add = tile_pre[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    if (base + k < n) out[base + k] += add;
}

__global__ void k_scatter(const int* __restrict__ atom_slot, int n, const int* __restrict__ start,
                          int* __restrict__ fill, int* __restrict__ unsorted) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int s = atom_slot[i];
  unsorted[start[s] + atomicAdd(&fill[s], 1)] = i;
}

// rank inside the cell: ascending atom index (NeighborList.cpp:104-117 fills
// each bucket while walking atoms in ascending order)
__global__ void k_rank(const int* __restrict__ unsorted, const int* __restrict__ atom_slot,
                       int n, const int* __restrict__ start, const int* __restrict__ count,
                       int* __restrict__ sorted) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int a = unsorted[p];
  int s = atom_slot[a];
  int lo = start[s], hi = lo + count[s];
  int r = 0;
  for (int q = lo; q < hi; q++) r += unsorted[q] < a;
  sorted[lo + r] = a;
}

__global__ void k_pos_build(const md_double4* __restrict__ pos, int n, float4* __restrict__ pb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  md_double4 p = pos[i];
  pb[i] = make_float4((float)p.x, (float)p.y, (float)p.z, __int_as_float((int)p.w));
}

// MODE 0: count (len[i] and maxima); MODE 1: write ELL rows.
template <int MODE>
__global__ void k_rows(RowWalker w, const md_double4* __restrict__ pos,
                       const float4* __restrict__ pb, int compact, float rv2, float box_f,
                       uint32_t* __restrict__ list, int* __restrict__ len, int ld,
                       int* __restrict__ counters) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.n) return;
  const float4 pi = pb[i];
  int full = 0, kept = 0;
  walk_row(w, pos, i, [&](int m, int ix, int iy, int iz) {
    full++;
    bool keep = true;
    if (compact) {
      float4 pm = pb[m];
      float dx = pi.x - (pm.x + (float)ix * box_f);
      float dy = pi.y - (pm.y + (float)iy * box_f);
      float dz = pi.z - (pm.z + (float)iz * box_f);
      keep = dx * dx + dy * dy + dz * dz < rv2;
    }
    if (keep) {
      if (MODE == 1) list[(size_t)kept * ld + i] = pack_entry(m, ix, iy, iz);
      kept++;
    }
  });
  if (MODE == 0) {
    len[i] = kept;
    // one atomic per warp for each counter
    const unsigned m = __activemask();
    const unsigned fmax_w = __reduce_max_sync(m, (unsigned)full);
    const unsigned kmax_w = __reduce_max_sync(m, (unsigned)kept);
    const unsigned ksum_w = __reduce_add_sync(m, (unsigned)kept);
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1) {
      atomicMax(&counters[1], (int)fmax_w);
      atomicMax(&counters[2], (int)kmax_w);
      atomicAdd((unsigned long long*)(counters + 4), (unsigned long long)ksum_w);
    }
  }
}

__global__ void k_ref_rows(RowWalker w, const md_double4* __restrict__ pos, int nls,
                           int* __restrict__ out, signed char* __restrict__ img) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.n) return;
  int* row = out + (size_t)i * nls;
  signed char* im = img ? img + (size_t)i * nls : nullptr;
  int count = 0;
  walk_row(w, pos, i, [&](int m, int ix, int iy, int iz) {
    if (count < nls) {
      row[count] = m;
      if (im) im[count] = (signed char)((ix + 1) * 9 + (iy + 1) * 3 + (iz + 1));
    }
    count++;
  });
  for (int k = count; k < nls; k++) {
    row[k] = -1;
    if (im) im[k] = 13;
  }
}

template <typename T>
cudaError_t grow(T*& p, long long& have, long long need) {
  if (need <= have && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  long long n = need > 0 ? need : 1;
  cudaError_t e = cudaMalloc(&p, sizeof(T) * (size_t)n);
  have = e == cudaSuccess ? n : 0;
  return e;
}

inline int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// cuTensorMapEncodeTiled of the CUDA driver API, looked up once through the runtime
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

int encode_tiled_2d(CUtensorMap* map, CUtensorMapDataType type, void* base, uint64_t dim0,
                    uint64_t dim1, uint64_t stride_bytes, uint32_t box0, uint32_t box1) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || stride_bytes % 16 != 0) return 0;
  cuuint64_t dims[2] = {(cuuint64_t)dim0, (cuuint64_t)dim1};
  cuuint64_t strides[1] = {(cuuint64_t)stride_bytes};
  cuuint32_t box[2] = {box0, box1};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, type, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 1 : 0;
}

// TMA descriptor of a compact list: a 2-D uint32 tensor of n atoms (x) by
// cap slots (y), row stride ld * 4 bytes; tiles of kListTileAtoms x
// kListTileSlots.  Out-of-range atoms and slots read as zero.
int encode_list_map(NeighborList& nl) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || (nl.ld * 4) % 16 != 0) return 0;
  cuuint64_t dims[2] = {(cuuint64_t)nl.n, (cuuint64_t)nl.cap};
  cuuint64_t strides[1] = {(cuuint64_t)nl.ld * 4};
  cuuint32_t box[2] = {kListTileAtoms, kListTileSlots};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(&nl.tmap, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, nl.list, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 1 : 0;
}

Grid make_grid_reference(double box_list, float rs) {
  Grid g{};
  g.periodic = 0;
  int cells = (int)((box_list / (double)rs) + 0.99f);  // NeighborList.cpp:21
  if (cells < 1) cells = 1;
  g.cells = cells;
  g.npos = box_list / 2;
  g.cs = (double)rs;
  g.box = box_list;
  g.box_f = 0.f;
  g.box_lo = 0.f;
  return g;
}

Grid make_grid_periodic(double L, float rs) {
  Grid g{};
  g.periodic = 1;
  int cells = (int)floor(L / (double)rs);
  if (cells < 3) cells = 1;
  g.cells = cells;
  g.npos = L * 0.5;
  g.cs = L / cells;
  g.box = L;
  g.box_f = (float)L;
  g.box_lo = (float)(L - (double)g.box_f);
  return g;
}

RowWalker make_walker(const NeighborList& nl) {
  RowWalker w;
  w.keys = nl.table.keys;
  w.count = nl.table.count;
  w.start = nl.table.start;
  w.sorted = nl.sorted;
  w.cell3 = nl.cell3;
  w.cap = nl.table.cap;
  w.n = nl.n;
  w.g = nl.grid;
  return w;
}

cudaError_t scan_exclusive(const int* in, int* out, int n, Scratch& sc, cudaStream_t st) {
  int tiles = blocks(n, kScanTile);
  if (tiles > kScanTile) return cudaErrorInvalidValue;
  if (sc.block_sums_cap < 2 * tiles + 2) {
    if (sc.block_sums) cudaFree(sc.block_sums);
    cudaError_t e = cudaMalloc(&sc.block_sums, sizeof(int) * (size_t)(2 * tiles + 2));
    if (e != cudaSuccess) return e;
    sc.block_sums_cap = 2 * tiles + 2;
  }
  int* sums = sc.block_sums;
  int* pre = sc.block_sums + tiles + 1;
  k_scan_tiles<<<tiles, kScanThreads, 0, st>>>(in, out, n, sums);
  k_scan_tiles<<<1, kScanThreads, 0, st>>>(sums, pre, tiles, nullptr);
  k_scan_add<<<tiles, kScanThreads, 0, st>>>(out, n, pre);
  return cudaGetLastError();
}

int list_build(NeighborList& nl, md_double4* pos, int n, const Grid& g, int compact, float rv,
               double rcut, Scratch& sc, int* d_status, cudaStream_t st, std::string& err) {
  if (n > kMaxAtoms) {
    err = "too many atoms for the packed list entry (2^26)";
    return -1;
  }
  nl.n = n;
  nl.grid = g;
  nl.compact = compact;
  nl.rv = rv;
  cudaError_t e;
  if (n > nl.n_alloc || !nl.cell3) {
    long long need = n > 0 ? n : 1;
    for (int** p : {&nl.atom_slot, &nl.unsorted, &nl.sorted}) {
      if (*p) cudaFree(*p);
      *p = nullptr;
      if ((e = cudaMalloc(p, sizeof(int) * need)) != cudaSuccess) return e;
    }
    if (nl.cell3) cudaFree(nl.cell3);
    if ((e = cudaMalloc(&nl.cell3, sizeof(int) * 4 * need)) != cudaSuccess) return e;
    if (nl.len) cudaFree(nl.len);
    if ((e = cudaMalloc(&nl.len, sizeof(int) * need)) != cudaSuccess) return e;
    if (nl.pos_build) cudaFree(nl.pos_build);
    if ((e = cudaMalloc(&nl.pos_build, sizeof(float4) * need)) != cudaSuccess) return e;
    nl.n_alloc = (int)need;
  }
  int cap = 64;
  while (cap < 2 * n + 16) cap <<= 1;
  if (cap > nl.table.cap) {
    for (int** p : {&nl.table.count, &nl.table.start, &nl.table.fill}) {
      if (*p) cudaFree(*p);
      *p = nullptr;
      if ((e = cudaMalloc(p, sizeof(int) * (size_t)cap)) != cudaSuccess) return e;
    }
    if (nl.table.keys) cudaFree(nl.table.keys);
    if ((e = cudaMalloc(&nl.table.keys, sizeof(unsigned long long) * (size_t)cap)) != cudaSuccess)
      return e;
    nl.table.cap = cap;
  }
  cap = nl.table.cap;
  cudaMemsetAsync(nl.table.keys, 0xFF, sizeof(unsigned long long) * (size_t)cap, st);
  cudaMemsetAsync(nl.table.count, 0, sizeof(int) * (size_t)cap, st);
  cudaMemsetAsync(nl.table.fill, 0, sizeof(int) * (size_t)cap, st);
  cudaMemsetAsync(sc.counts, 0, sizeof(int) * 8, st);
  const int T = 256;
  if (n > 0) {
    k_cell_assign<<<blocks(n, T), T, 0, st>>>(pos, n, g, nl.cell3, nl.table.keys, nl.table.count,
                                              cap, nl.atom_slot, sc.counts, d_status);
    k_pos_build<<<blocks(n, T), T, 0, st>>>(pos, n, nl.pos_build);
  }
  if ((e = scan_exclusive(nl.table.count, nl.table.start, cap, sc, st)) != cudaSuccess) return e;
  if (n > 0) {
    k_scatter<<<blocks(n, T), T, 0, st>>>(nl.atom_slot, n, nl.table.start, nl.table.fill,
                                          nl.unsorted);
    k_rank<<<blocks(n, T), T, 0, st>>>(nl.unsorted, nl.atom_slot, n, nl.table.start,
                                       nl.table.count, nl.sorted);
  }
  RowWalker w = make_walker(nl);
  // compact filter radius, widened by a margin for FP32 rounding of the
  // build-time positions; the skin test uses rv itself
  float margin = (float)(1e-6 * (fabs(g.box) + rv) + 1e-6);
  float rv_keep = rv + margin;
  float rv2 = compact ? rv_keep * rv_keep : 0.f;
  if (n > 0)
    k_rows<0><<<blocks(n, 128), 128, 0, st>>>(w, pos, nl.pos_build, compact, rv2, g.box_f,
                                              nullptr, nl.len, n, sc.counts);
  int hc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int status = 0;
  cudaMemcpyAsync(hc, sc.counts, sizeof(hc), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  if (status & (ST_CELL_OVERFLOW | ST_NONFINITE)) {
    err = (status & ST_NONFINITE) ? "non-finite position at list build"
                                  : "cell grid out of range at list build";
    return -1;
  }
  nl.maxcell = hc[0];
  nl.nlargest = hc[1];
  {
    unsigned long long ent;
    memcpy(&ent, hc + 4, sizeof(ent));
    nl.entries = (long long)ent;
  }
  long long nls = (long long)hc[0] * 27;
  if (nls > n - 1) nls = n - 1;
  if (nls < 0) nls = 0;
  nl.nlistsize = (int)nls;
  nl.max_len = hc[2];
  int need_cap = hc[2] > 0 ? hc[2] : 1;
  if (compact) need_cap = (int)(need_cap * nl.headroom) + 8;  // room for skin refreshes
  nl.ld = ((n > 0 ? n : 1) + 31) / 32 * 32;
  long long elems = (long long)need_cap * nl.ld;
  if ((e = grow(nl.list, nl.list_elems, elems)) != cudaSuccess) return e;
  nl.cap = need_cap;
  nl.tmap_ok = compact && n > 0 ? encode_list_map(nl) : 0;
  if (n > 0)
    k_rows<1><<<blocks(n, 128), 128, 0, st>>>(w, pos, nl.pos_build, compact, rv2, g.box_f,
                                              nl.list, nl.len, nl.ld, sc.counts);
  double rc = rcut;
  nl.trip_dist = compact ? 0.5 * ((double)rv - rc) - (double)margin : 1e300;
  nl.rv2_keep = rv2;
  if (!nl.skin) {
    if ((e = cudaMalloc(&nl.skin, sizeof(int) * 4)) != cudaSuccess) return e;
    // [3], the trip count, is cleared by its reader after each build: zero it once here
    cudaMemsetAsync(nl.skin, 0, sizeof(int) * 4, st);
  }
  cudaMemsetAsync(nl.skin, 0, sizeof(int) * 3, st);
  return (int)cudaGetLastError();
}

int list_reference_rows(const NeighborList& nl, const md_double4* pos, int* d_out,
                        signed char* d_img, cudaStream_t st) {
  if (nl.n <= 0 || nl.nlistsize <= 0) return 0;
  RowWalker w = make_walker(nl);
  k_ref_rows<<<blocks(nl.n, 128), 128, 0, st>>>(w, pos, nl.nlistsize, d_out, d_img);
  return (int)cudaGetLastError();
}

void list_free(NeighborList& nl) {
  for (void* p : {(void*)nl.table.keys, (void*)nl.table.count, (void*)nl.table.start,
                  (void*)nl.table.fill, (void*)nl.atom_slot, (void*)nl.cell3,
                  (void*)nl.unsorted, (void*)nl.sorted, (void*)nl.list, (void*)nl.len,
                  (void*)nl.pos_build, (void*)nl.skin})
    if (p) cudaFree(p);
  nl = NeighborList();
}

}  // namespace mdgb
