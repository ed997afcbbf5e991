// Device-side walk over a full candidate row (common/NeighborList.cpp:131-168):
// the 27 cells around an atom's build-time cell in the order dx, dy, dz =
// -1..1, each cell's atoms in ascending index, the atom itself skipped.
#pragma once
#include "md_internal.h"

namespace mdgb {

constexpr unsigned long long kEmptyKey = ~0ULL;

__host__ __device__ __forceinline__ unsigned long long cell_key(int cx, int cy, int cz) {
  return ((unsigned long long)(cx + 1) << 42) | ((unsigned long long)(cy + 1) << 21) |
         (unsigned long long)(cz + 1);
}
__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 31;
  x *= 0x9e3779b97f4a7c15ULL;
  x ^= x >> 29;
  return x;
}
__device__ __forceinline__ int table_find(const unsigned long long* keys, int cap,
                                          unsigned long long key) {
  unsigned h = (unsigned)(mix64(key) & (unsigned long long)(cap - 1));
  for (int probe = 0; probe < cap; probe++) {
    unsigned long long k = keys[h];
    if (k == key) return (int)h;
    if (k == kEmptyKey) return -1;
    h = (h + 1) & (unsigned)(cap - 1);
  }
  return -1;
}

// Minimum image of m seen from i in a periodic box with a single cell.
__device__ __forceinline__ int min_image(double xi, double xm, double L) {
  double d = xi - xm;
  return d > 0.5 * L ? 1 : (d < -0.5 * L ? -1 : 0);
}

// visit(m, ix, iy, iz) for every candidate of row i, in reference order.
template <typename F>
__device__ __forceinline__ void walk_row(const RowWalker& w, const md_double4* pos, int i,
                                         F&& visit) {
  if (w.g.periodic && w.g.cells == 1) {
    md_double4 pi = pos[i];
    for (int m = 0; m < w.n; m++) {
      if (m == i) continue;
      md_double4 pm = pos[m];
      visit(m, min_image(pi.x, pm.x, w.g.box), min_image(pi.y, pm.y, w.g.box),
            min_image(pi.z, pm.z, w.g.box));
    }
    return;
  }
  const int4 c4 = reinterpret_cast<const int4*>(w.cell3)[i];
  const int cx = c4.x, cy = c4.y, cz = c4.z;
  const int cells = w.g.cells;
  for (int dx = -1; dx < 2; dx++)
    for (int dy = -1; dy < 2; dy++)
      for (int dz = -1; dz < 2; dz++) {
        int nc[3] = {cx + dx, cy + dy, cz + dz};
        int im[3] = {0, 0, 0};
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
        if (out) continue;
        int s = table_find(w.keys, w.cap, cell_key(nc[0], nc[1], nc[2]));
        if (s < 0) continue;
        const int a = w.start[s], b = a + w.count[s];
        for (int q = a; q < b; q++) {
          int m = w.sorted[q];
          if (m != i) visit(m, im[0], im[1], im[2]);
        }
      }
}

// Is j in the full candidate row of k (27-cell adjacency of build-time
// cells)?  img receives the periodic image of j in k's row, as walk_row
// produces it.  Periodic boxes need at least 3 cells per axis here.
__device__ __forceinline__ bool in_row(const int* cell3, const Grid& g, int k, int j,
                                       int* img) {
  if (j == k) return false;
  const int4 k4 = reinterpret_cast<const int4*>(cell3)[k], j4 = reinterpret_cast<const int4*>(cell3)[j];
  const int ck3[3] = {k4.x, k4.y, k4.z}, cj3[3] = {j4.x, j4.y, j4.z};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    int ck = ck3[d], cj = cj3[d];
    img[d] = 0;
    if (!g.periodic) {
      int dd = cj - ck;
      if (dd < -1 || dd > 1 || cj < 0 || cj >= g.cells) return false;
    } else {
      int s = cj - ck;
      if (s > 1) s -= g.cells;
      if (s < -1) s += g.cells;
      if (s < -1 || s > 1) return false;
      int nc = ck + s;
      img[d] = nc < 0 ? -1 : (nc >= g.cells ? 1 : 0);
    }
  }
  return true;
}

}  // namespace mdgb
