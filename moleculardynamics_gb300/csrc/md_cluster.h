// Cell-cluster neighbour structure of the precision form in periodic boxes.
//
// At every list build the atoms of each replica are sorted by dense cell
// (x slowest, z fastest; atoms of a cell in ascending original index) and the
// whole state is permuted into that order.  A segment is a run of consecutive
// cells of one z-column holding at most one block's worth of atoms (cut
// greedily at the build); its thread block stages the positions of the 9
// columns around it, over cells cz0-1 .. cz1+1 with periodic images, in
// shared memory ("pieces", in the stencil order dx, dy, dz of
// common/NeighborList.cpp:142-168).  An atom's 27-cell candidate row is then
// 9 contiguous ranges of the staged array, in the reference's candidate
// order, and its compact row stores 16-bit offsets into it.  Rows are
// slot-major (rows[k * ld + p]); the force kernel streams a segment's rows
// into shared memory by TMA in tiles of 16 slots.  Boxes under 3 cells per
// edge are one segment staging the whole replica; pairs then take the
// minimum image.  Several independent replicas (each its own periodic box)
// share one structure: their atoms, cells and segments are contiguous
// ranges, and one launch covers all of them.
#pragma once
#include <vector>

#include "md_integrate.h"
#include "md_internal.h"

namespace mdgb {

struct ClusterReplica {
  int atom0, n;      // atoms [atom0, atom0 + n) of the state
  int cell0;         // first global dense cell
  int col0;          // first global z-column
  int G;             // cells per edge (1: one cell, minimum image)
  int pad;
  double L, cs;      // box edge and cell size
  double invL, invcs;  // their reciprocals (screening of the cell divisions)
  float Lf, Llo;     // L = Lf + Llo
};

struct ClusterPiece {
  int src, count, dst;
  signed char ix, iy, iz, pad;
};
constexpr int kClusterMaxPieces = 27;
constexpr int kClusterMaxZ = 64;            // cells per segment
constexpr int kClusterMaxStaged = 11264;    // staged atoms per segment (176 KB)
constexpr int kClusterTileSlots = 16;       // row slots per TMA tile

struct ClusterSegment {
  int rep, cx, cy, cz0, cz1;
  int p0, p1;        // sorted atoms of the segment's cells
  int staged;        // atoms staged in shared memory
  int npieces;
  int self0;         // staged offset of the segment's first own atom
  int img;           // some piece carries a periodic image
  int group[10];     // first piece of each (dx, dy) group (9 groups + end)
  ClusterPiece piece[kClusterMaxPieces];
};

struct ClusterList {
  int nrep = 0, natoms = 0;
  std::vector<ClusterReplica> h_rep;
  ClusterReplica* rep = nullptr;
  int nseg = 0, seg_alloc = 0;
  ClusterSegment* seg = nullptr;
  int ncells = 0, ncols = 0, cells_alloc = 0;
  int *count = nullptr, *start = nullptr, *fill = nullptr, *segidx = nullptr;
  int n_alloc = 0;
  int* cell = nullptr;                            // global cell of each stored atom
  int *unsorted = nullptr, *perm = nullptr;       // perm[p] = storage index before the sort
  int *orig = nullptr, *itmp = nullptr;           // original index of each stored atom
  uint16_t* rows = nullptr;                       // rows[k * ld + p]: staged offsets
  uint16_t* len = nullptr;
  long long rows_elems = 0;
  int ld = 0, cap = 0;
  float4* pos_build = nullptr;
  // shadow buffers of the permutation (same sizes as the state arrays)
  md_double4* pos_tmp = nullptr;
  double* v3_tmp[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // skin flags: [0..2] trip flag of step t at t % 3 (the force kernel of
  // step t reads [t % 3], the Gear update sets [(t + 1) % 3], and [(t + 2) % 3]
  // is cleared); [3] refresh overflow (sticky until the next build);
  // [4] refreshes done
  int* skin = nullptr;
  float rv = 0.f, rv2 = 0.f, headroom = 1.25f;
  double trip_dist = 0;
  int max_staged = 0, maxlen = 0, maxcell = 0;
  long long entries = 0;
  int Z = kClusterMaxZ;                           // cells per segment (upper bound)
  int block = 128;                                // threads per segment block (<= 224)
  int stage_cap = kClusterMaxStaged;              // staged atoms per segment (soft cap)
  int row_loads = 1;                              // 1 block TMA tiles, 2 register prefetch,
                                                  // 3 per-warp TMA tiles
  int grouped = 0;                                // rows grouped by eight slots with byte
                                                  // offsets (the register-prefetch scheme):
                                                  // rows[((k / 8) ld + p) 8 + k % 8] = 16 q
  CUtensorMap rmap;                               // TMA map of rows: {ld atoms, cap slots}
  CUtensorMap rmap_w;                             // the same with per-warp boxes
  int rmap_ok = 0;
  int* counters = nullptr;                        // device: max staged, max len, entries, max cell
  int* sched = nullptr;                           // device: persistent kernel's work counters
  bool built = false;
  int version = 0;  // counts builds (each may change the order)
};

// Builds (or rebuilds) the structure for the replicas in `reps` (n and L
// set; the rest is filled in).  Positions are wrapped into each box and the
// state (*pos and the five *v3 arrays: vel, acc, b, c, force; any may be
// NULL) is permuted into cell order by swapping in the shadow buffers.
// posf receives the FP32 copy of the permuted positions.  Returns a
// cudaError_t, or -1 with err set.
int cluster_build(ClusterList& cl, const std::vector<ClusterReplica>& reps, float rv, double rcut,
                  md_double4** pos, double** v3[5], float4* posf, Scratch& sc, int* d_status,
                  cudaStream_t st, std::string& err);
void cluster_free(ClusterList& cl);

// Gear correct (this step) + predict (next step) fused into the force
// kernel: the next positions go to pos_next / posf_next (the current ones are
// still read by other blocks), vel/acc/b/c are updated in place.
struct ClusterGearArgs {
  md_double4* pos_next;
  float4* posf_next;
  double *vel, *acc, *b, *c;
  GearCoef k;
  double inv_mass[3];
  float trip2;       // squared skin displacement (< 0: trip every step)
  bool correct_only = false;  // stop after the correct (forces also go to f3)
};

struct ClusterForceArgs {
  const ClusterList* cl;
  const float4* posf;
  const md_double4* pos;
  double* f3;        // forces out (unused when gear is set, unless correct_only)
  int step;          // MD step t of this evaluation (skin flag rotation)
  double rcutsq;
  Species sp;
  int all_ng;
  double* epart;     // 3 doubles per segment block (energy)
  int* status;       // ST_TMA_TIMEOUT / ST_NONFINITE
  const ClusterGearArgs* gear;  // NULL: forces only
  int* skin = nullptr;          // skin flags (NULL: the list's own)
  int wait_limit = 1 << 20;     // polls of a bounded mbarrier wait (0: give up at once)
};
void launch_lj_cluster(const ClusterForceArgs& a, bool energy, cudaStream_t st);
// inv[orig[p]] = p
void launch_invert(const int* orig, int* inv, int n, cudaStream_t st);
// Transfers between the cell-ordered state and a caller array in its own
// order that the device reaches directly (pinned host memory), element by
// element in the caller's order: dst[width inv[i] + d] = host[width i + d],
// and back.
void launch_gather_host(const double* host, double* dst, const int* inv, int n, int width,
                        cudaStream_t st);
void launch_scatter_host(const double* src, double* host, const int* inv, int n, int width,
                         cudaStream_t st);
// flag |= 1 when some atom is not of the NG species
void launch_species_check(const md_double4* pos, int n, int* flag, cudaStream_t st);
int cluster_blocks(const ClusterList& cl);
// Largest stage cap (staged atoms per segment) at which the fused every-step
// launch of `threads`-thread blocks on row scheme `row_loads` keeps the
// blocks per SM that its registers allow (the kernels' shared-memory limits
// must have been raised: any cluster_build does it).
int cluster_occupancy_cap(int threads, int row_loads, bool all_ng);

// Reference-layout rows (common/NeighborList.cpp:119-177) of atoms in their
// original numbering: out[o * nlistsize + k], -1 padded; images as
// md_neighbor_list reports them; *d_nlargest (zeroed by the caller) receives
// the longest row (nlargestsize).  d_out may be NULL.  Single replica.
int cluster_reference_rows(const ClusterList& cl, const md_double4* pos, int nlistsize,
                           int* d_out, signed char* d_img, int* d_nlargest, cudaStream_t st);

// out3[3k..3k+2] = sum of epart over the segments of replica k (the
// per-segment energies of an energy launch of launch_lj_cluster)
void launch_rep_energy(const ClusterList& cl, const double* epart, double* out3,
                       cudaStream_t st);

// out[orig[p]] = in[p] for arrays of `width` doubles per atom
void launch_unpermute(const double* in, double* out, const int* orig, int n, int width,
                      cudaStream_t st);
// out[p] = in[orig[p]]
void launch_permute_in(const double* in, double* out, const int* orig, int n, int width,
                       cudaStream_t st);

}  // namespace mdgb
