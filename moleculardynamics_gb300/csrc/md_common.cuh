// Shared device definitions of the GB300 MD step engine.
//
// Constants are the reference's float literals (common/Constants.h:13-79) and
// are promoted to double exactly where the reference promotes them, so that
// the FP64 kernels evaluate the same expressions as the reference CPU path
// (cpumd is built with real = double, cpu/cpumd/cpumd.vcproj:46).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mdgb {

// Positions on the device use the reference's real4 layout (x, y, z, type),
// 32-byte aligned so that one atom is one 256-bit load.
typedef double4_32a md_double4;

// species indices, common/Constants.h:13-15
constexpr int SP_N = 0, SP_O = 1, SP_NG = 2;

#define MD_reN 1.097f
#define MD_reO 1.2075f
#define MD_reNO 1.15f
#define MD_reNvdw 3.72f
#define MD_reOvdw 3.31f
#define MD_reNOvdw 3.51f
#define MD_sigNvdw 3.31f
#define MD_deN 941.4e-4f
#define MD_deO 493.55309e-4f
#define MD_deNO 626.734e-4f
#define MD_betaN 2.71009f
#define MD_betaO 2.2478f
#define MD_betaNO 2.24068f
#define MD_CUTOFF_RIJ (15 * MD_sigNvdw)
#define MD_CUTOFF_RIJSQ (225 * MD_sigNvdw * MD_sigNvdw)
#define MD_GEAR1 0.15833333333333333333333333333333f
#define MD_GEAR2 0.75f
#define MD_GEAR3 0.5f
#define MD_GEAR4 0.08333333333333333333333333333333f
#define MD_S 2.0f
#define MD_GM 0.3f
#define MD_GMSQ 0.09f
#define MD_ALFAV 3.0f
#define MD_ALFAVSQ 9.0f
#define MD_ALFA 2.0f
#define MD_R0 1.3f
#define MD_LAMDA3 1.33f
#define MD_C 25.f
#define MD_D 4.0417f
#define MD_H 0.0f
#define MD_KB 8.314e-7f

// Lennard-Jones parameters of the NG slot and the three masses
// (common/Constants.h:36-43,55-57); floats, promoted where used.
struct Species {
  float sig[3];  // indexed by the "select" species of LennardJones.h:65-86
  float eps[3];
  float mass[3];
};

// Packed neighbour entry: atom index in bits 0..25, periodic image of the
// neighbour in bits 26..31 (2 bits per axis: 0 -> 0, 1 -> +1, 3 -> -1).
// Without a periodic box an entry is the plain index.
constexpr uint32_t kIndexBits = 26;
constexpr uint32_t kIndexMask = (1u << kIndexBits) - 1u;
constexpr int kMaxAtoms = 1 << kIndexBits;

__host__ __device__ __forceinline__ uint32_t pack_entry(int j, int ix, int iy, int iz) {
  return (uint32_t)j | ((uint32_t)(ix & 3) << 26) | ((uint32_t)(iy & 3) << 28) |
         ((uint32_t)(iz & 3) << 30);
}
__host__ __device__ __forceinline__ int entry_index(uint32_t e) { return (int)(e & kIndexMask); }
__host__ __device__ __forceinline__ int entry_img(uint32_t e, int axis) {
  int f = (int)((e >> (26 + 2 * axis)) & 3u);
  return (f ^ 2) - 2;
}

// TMA tile of a compact neighbour list: 128 atoms x 16 slots of uint32.
constexpr int kListTileAtoms = 128;
constexpr int kListTileSlots = 16;

// Cell-grid geometry of one list build.
struct Grid {
  int periodic;   // 0: reference box (NeighborList.cpp:19-27), 1: periodic cube
  int cells;      // cells per axis; periodic boxes below 3 cells use 1 (minimum image)
  double npos;    // half box
  double cs;      // cell size
  double box;     // reference: boxSizeList; periodic: edge L
  float box_f;    // L rounded to float (FP32 image shifts)
  float box_lo;   // L - box_f, added to FP32 image shifts
};

// ---- exact-rounding FP64 helpers (no FMA contraction) ----
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xdiv(double a, double b) { return __ddiv_rn(a, b); }

// squared norm evaluated as (x*x + y*y) + z*z, as the reference writes it
__device__ __forceinline__ double norm2_exact(double x, double y, double z) {
  return xadd(xadd(xmul(x, x), xmul(y, y)), xmul(z, z));
}

}  // namespace mdgb
