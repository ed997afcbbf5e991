// Internal host-side interfaces shared by the engine's translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "md_common.cuh"

namespace mdgb {

// Device status word bits (set by kernels, read by the host).
enum : int {
  ST_NONFINITE = 2,       // NaN/inf seen in positions or forces
  ST_CELL_OVERFLOW = 4,   // hash table full or cell coordinate out of range
  ST_XI_MISSING = 8,      // bond-order pass 2 needed a xi pass 1 did not make
  ST_WALL_HIT = 16,       // a wall reflection happened (cpu/common/Device.cpp:86-118)
  ST_TMA_TIMEOUT = 32,    // a bounded wait on a TMA transfer ran out
};

// Cell structure of one list build (open-addressing table of cells).
struct CellTable {
  unsigned long long* keys = nullptr;  // 0xFFFF... = empty
  int* count = nullptr;
  int* start = nullptr;
  int* fill = nullptr;
  int cap = 0;  // power of two
};

// One neighbour list: atoms [0, n) of the engine, rows in ELL slot-major
// layout list[k * n + i] of packed entries (md_common.cuh).
struct NeighborList {
  int n = 0;
  Grid grid{};
  CellTable table;
  int* atom_slot = nullptr;    // table slot of each atom's cell
  int* cell3 = nullptr;        // build-time cell coordinates (x, y, z, unused: 4 ints per atom)
  int* unsorted = nullptr;
  int* sorted = nullptr;       // atoms grouped by slot, ascending inside a cell
  uint32_t* list = nullptr;
  int* len = nullptr;
  int ld = 0;                  // leading dimension: list[k * ld + i], ld = n rounded up to 32
  int cap = 0;                 // slots per row allocated
  CUtensorMap tmap;            // TMA descriptor of the list (compact lists)
  int tmap_ok = 0;
  long long list_elems = 0;    // allocated list entries
  float4* pos_build = nullptr; // FP32 positions at build time (skin check)
  int compact = 0;             // 1: rows filtered at radius rv; 0: full candidate rows
  float rv = 0.f;
  double trip_dist = 0;        // an atom displaced by more than this trips the list
  float rv2_keep = 0.f;        // squared filter radius (rv plus FP32 margin)
  float headroom = 1.25f;      // compact row capacity / longest row at build
  // skin flags: [0], [1] trip flag of even / odd steps, [2] refresh overflow
  // (sticky until the next build), [3] refreshes done
  int* skin = nullptr;
  // host copies of the last build's sizes
  int maxcell = 0, nlargest = 0, nlistsize = 0, max_len = 0;
  long long entries = 0;         // total kept entries
  int n_alloc = 0;
};

// Scratch shared by reductions.
struct Scratch {
  double* dpart = nullptr;  // per-block partial sums
  int dpart_cap = 0;
  unsigned long long* umax = nullptr;  // 4 max slots
  int* counts = nullptr;               // 4 int counters
  int* block_sums = nullptr;
  int block_sums_cap = 0;
};

// ---- list module (md_neighbor.cu) ----
// Builds cells, ordering and rows of `nl` for atoms [0, n) of pos.  With
// grid.periodic the positions are wrapped into the box (pos is modified).
// Returns a cudaError_t, or -1 on a status failure recorded in *status_h.
int list_build(NeighborList& nl, md_double4* pos, int n, const Grid& g, int compact, float rv,
               double rcut, Scratch& sc, int* d_status, cudaStream_t st, std::string& err);
// Reference-layout rows (NeighborList.cpp:119-177): out[i*nlistsize + k], -1 padded.
int list_reference_rows(const NeighborList& nl, const md_double4* pos, int* d_out,
                        signed char* d_img, cudaStream_t st);
void list_free(NeighborList& nl);
Grid make_grid_reference(double box_list, float rs);
// 2-D tiled TMA descriptor (no swizzle, zero fill out of range); 1 on success
int encode_tiled_2d(CUtensorMap* map, CUtensorMapDataType type, void* base, uint64_t dim0,
                    uint64_t dim1, uint64_t stride_bytes, uint32_t box0, uint32_t box1);
// exclusive prefix sum of n ints (n <= 2^24)
cudaError_t scan_exclusive(const int* in, int* out, int n, Scratch& sc, cudaStream_t st);
Grid make_grid_periodic(double L, float rs);

// Walk context handed to kernels that iterate full candidate rows.
struct RowWalker {
  const unsigned long long* keys;
  const int* count;
  const int* start;
  const int* sorted;
  const int* cell3;
  int cap;
  int n;
  Grid g;
};
RowWalker make_walker(const NeighborList& nl);

}  // namespace mdgb
