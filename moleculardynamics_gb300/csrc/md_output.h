// Device side of the run's outputs: animation frames (common/Results.cpp:12-31,
// 51-86) and the N-O pair list of the many-body atoms (common/Results.cpp:88-118).
#pragma once
#include <cuda_runtime.h>

#include "md_common.cuh"

namespace mdgb {

// One animation frame as the reference's pushAnim keeps it: positions as
// n x float4 (x, y, z, type) followed by velocities as n x float3, each a
// (float) conversion of the FP64 state, in the caller's numbering (orig maps
// a stored atom to it; NULL: stored in the caller's order).
void launch_anim_pack(const md_double4* pos, const double* vel, const int* orig, int n,
                      float* out, cudaStream_t st);

// Pairs i < j < n of different species whose FP64 distance is below
// 2 reNO, in the reference's order (i, then j, ascending); pairs[2k],
// pairs[2k + 1] for k < min(count, capacity).  Synchronous.  Returns a CUDA
// error code (0: success).
int tail_pairs(const md_double4* pos, int n, int* pairs, int capacity, int* count,
               cudaStream_t st);

}  // namespace mdgb
