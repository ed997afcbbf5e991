// Launch interface of the force kernels (md_forces.cu).
#pragma once
#include "md_internal.h"

namespace mdgb {

struct ForceArgs {
  const md_double4* pos;
  const float4* posf;   // FP32 copy (precision form)
  double* f3;
  int n;
  uint32_t* list;       // compact rows (rewritten per atom after a skin trip)
  int* len;
  int ld;               // list[k * ld + i]
  const CUtensorMap* tmap;  // TMA descriptor of the list (NULL: no TMA kernel)
  int all_ng;           // every atom is of the NG species
  int* status;
  RowWalker walker;     // full rows, walked when the skin is tripped
  int* skin;            // NeighborList::skin
  int parity;           // step parity: skin[parity] is this step's trip flag
  int cap;              // compact row capacity
  float rv2;            // compact filter radius squared
  float4* pos_build;    // skin reference positions
  double rcutsq;
  Species sp;
  double* epart;        // 3 doubles per block when energy is requested
  int wait_limit = 1 << 20;  // polls of a bounded mbarrier wait (0: give up at once)
};

struct MbArgs {
  const md_double4* pos;
  const float4* posf;
  double* f3;
  int n;                // many-body atoms [0, n)
  const uint32_t* list; // full candidate rows, list[k * ld + i]
  const int* len;
  int ld;
  Grid grid;
  const int* cell3;     // build-time cells of the many-body list
  const int* ref_rows;  // or: rows in the reference layout (membership by scan)
  int ref_nls;
  int ref_nlargest;
  double rcutsq;
  int ljexist;          // accumulate onto F (BondOrderFuncs.h:325-336)
  uint32_t* sl;         // short list scratch (cap x n)
  int* slen;
  void* xsi;            // per (i, slot), T: pass 2's factor va E / (4 (1 + xi_ij)^2)
  void* xsj;            // and va E / (4 (1 + xi_ji)^2), NaN where pass 1 skipped the pair
  int* missing;
  const int* run_if = nullptr;  // force launches only: return at once unless *run_if != 0
  double* epart1;       // 2 doubles per pass-1 block
  double* epart2;       // 1 double per pass-2 block
  double* eatom = nullptr;  // energy launches: per-atom energy (sum over j of half the pair)
};

void launch_lj(const ForceArgs& a, bool fp32, bool energy, cudaStream_t st);
void launch_mb(const MbArgs& a, bool fp32, bool energy, cudaStream_t st);
int lj_blocks(int n);
int mb_blocks(int n);

}  // namespace mdgb
