// Force kernels: Lennard-Jones (cpu/common/LennardJones.h) and the bond-order
// many-body term (cpu/common/BondOrderFuncs.h).
//
// LJ, FP64 ("plain"): one thread per atom walks its compact row in the
// reference's candidate order and evaluates every in-range pair with the
// reference's roundings (no FMA contraction), so that forces are bit-identical
// to the reference on the same positions and list.
// LJ, FP32 (precision form): same rows; pair arithmetic in FP32 from the FP32
// position copy; pairs within 1e-5 of the cutoff are re-tested in FP64 so the
// pair set equals the FP64 one; per-atom sums are FP32 chunks of 16 pairs
// folded into a compensated (Kahan) FP32 pair (hi, lo), stored as FP64.
// Bond order: a short list per atom (candidates within rcut now), then
//   pass 1: one warp per atom i, one lane per pair (i, j); the lane loops over
//           the third bodies m of i's short list (BondOrderFuncs.h:12-143,
//           242-278) and stores xi_ij, xi_ji and Va_ij per (i, slot);
//   pass 2: one warp per atom k, one lane per i of k's short list; the lane
//           loops over j of i's short list that lie in k's candidate row and
//           adds k's third-body force (BondOrderFuncs.h:148-237, 339-393).
// Lane sums are combined with warp shuffles.
#include <type_traits>
#include <cmath>

#include "md_forces.h"
#include "md_neighbor.cuh"
#include "md_potential.cuh"
#include "md_tma.cuh"

namespace mdgb {

namespace {

// current FP32 position of atom j (the FP32 copy when there is one)
__device__ __forceinline__ float4 cur_pos(const md_double4* pos, const float4* posf, int j) {
  if (posf) return posf[j];
  const md_double4 p = pos[j];
  return make_float4((float)p.x, (float)p.y, (float)p.z, __int_as_float((int)p.w));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of NV doubles over the block, written to out[NV * blockIdx.x + k].
template <int NV>
__device__ __forceinline__ void block_partial(double (&v)[NV], double* out) {
  __shared__ double sm[NV][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double x = warp_sum(v[k]);
    if (lane == 0) sm[k][warp] = x;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double x = lane < nw ? sm[k][lane] : 0.0;
      x = warp_sum(x);
      if (lane == 0) out[NV * blockIdx.x + k] = x;
    }
  }
}

// ------------------------------------------------------------------ LJ FP64
template <bool ENERGY>
__global__ void __launch_bounds__(128)
    k_lj_fp64(const md_double4* __restrict__ pos, double* __restrict__ f3, int n, int ld,
              uint32_t* __restrict__ list, int* __restrict__ len, RowWalker w, int* skin,
              int parity, int cap, float rv2, float4* __restrict__ pos_build, double rcutsq,
              Species sp, double* __restrict__ epart) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ev[3] = {0.0, 0.0, 0.0};
  if (i < n) {
    const md_double4 pi = pos[i];
    const int ti = (int)pi.w;
    const double box = w.g.box;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    // the species-pair constants of LennardJones.h:12-30, once per thread
    double sq[3], cn[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {
      sq[t] = lj_sigsq(sp.sig[t]);
      cn[t] = lj_con(sp.eps[t], sq[t]);
    }
    auto visit = [&](int j, int ix, int iy, int iz, bool img) {
      const md_double4 pj = pos[j];
      double xj = pj.x, yj = pj.y, zj = pj.z;
      if (img) {
        xj = xadd(xj, (double)ix * box);
        yj = xadd(yj, (double)iy * box);
        zj = xadd(zj, (double)iz * box);
      }
      const double ijx = xsub(pi.x, xj), ijy = xsub(pi.y, yj), ijz = xsub(pi.z, zj);
      const double r2 = norm2_exact(ijx, ijy, ijz);
      if (r2 >= rcutsq) return;
      const int tj = (int)pj.w;
      if (tj == SP_NG || ti == SP_NG) {
        const int sel = lj_select(ti, tj);
        const double sig = sp.sig[sel], eps = sp.eps[sel];
        const double sigsq = sel == 0 ? sq[0] : (sel == 1 ? sq[1] : sq[2]);
        const double con = sel == 0 ? cn[0] : (sel == 1 ? cn[1] : cn[2]);
        const double fij = lj_pair_exact_c(fx, fy, fz, __dsqrt_rn(r2), ijx, ijy, ijz, sigsq, con);
        if (ENERGY) {
          // common/DebugCalculations.cpp:199-201 per ordered pair, restricted
          // to the force's pairs; shifted by its value at the cutoff
          double sr2 = xdiv(xmul(sig, sig), r2);
          double sr6 = xmul(xmul(sr2, sr2), sr2);
          double e = xmul(xmul(2.0, eps), xsub(xmul(sr6, sr6), sr6));
          double src2 = xdiv(xmul(sig, sig), rcutsq);
          double src6 = xmul(xmul(src2, src2), src2);
          ev[0] += e;
          ev[1] += e - xmul(xmul(2.0, eps), xsub(xmul(src6, src6), src6));
          ev[2] += 0.5 * (ijx * (ijx * fij) + ijy * (ijy * fij) + ijz * (ijz * fij));
        }
      }
    };
    const bool tripped = (skin[parity] | skin[2]) != 0;
    if (!tripped) {
      const int L = len[i];
      for (int k = 0; k < L; k++) {
        const uint32_t e = list[(size_t)k * ld + i];
        visit(entry_index(e), entry_img(e, 0), entry_img(e, 1), entry_img(e, 2), (e >> 26) != 0);
      }
    } else {
      // skin exceeded: walk the full candidate row (the reference's row,
      // same order) and refresh this atom's compact row at the current
      // positions, so that the following steps use the compact row again
      const float4 pc = cur_pos(pos, (const float4*)nullptr, i);
      int kept = 0;
      walk_row(w, pos, i, [&](int m, int ix, int iy, int iz) {
        visit(m, ix, iy, iz, w.g.periodic && (ix | iy | iz));
        const float4 pm = cur_pos(pos, (const float4*)nullptr, m);
        const float dx = pc.x - (pm.x + (float)ix * w.g.box_f);
        const float dy = pc.y - (pm.y + (float)iy * w.g.box_f);
        const float dz = pc.z - (pm.z + (float)iz * w.g.box_f);
        if (dx * dx + dy * dy + dz * dz < rv2) {
          if (kept < cap) list[(size_t)kept * ld + i] = pack_entry(m, ix, iy, iz);
          kept++;
        }
      });
      if (kept > cap) atomicOr(&skin[2], 1);
      len[i] = kept < cap ? kept : cap;
      pos_build[i] = pc;
      if (i == 0) atomicAdd(&skin[3], 1);
    }
    if (i == 0) skin[parity ^ 1] = 0;  // the next step's flag starts clear
    f3[3 * i] = fx;
    f3[3 * i + 1] = fy;
    f3[3 * i + 2] = fz;
  }
  if (ENERGY) block_partial<3>(ev, epart);
}

// ------------------------------------------------------------------ LJ FP32
__device__ __forceinline__ void kahan(float& hi, float& lo, float x) {
  float y = x - lo;
  float t = hi + y;
  lo = (t - hi) - y;
  hi = t;
}

// Is the FP32 pair (i, j) inside rcut?  Pairs within a relative 1e-5 band of
// the cutoff are decided in FP64 exactly as the FP64 path decides them.
__device__ __forceinline__ bool lj_inside(float r2, float rc_lo, float rc_hi,
                                          const md_double4* pos, int i, int j, bool img,
                                          int ix, int iy, int iz, const Grid& g,
                                          double rcutsq) {
  if (r2 >= rc_hi) return false;
  if (r2 <= rc_lo) return true;
  const md_double4 a = pos[i], b = pos[j];
  double xj = b.x, yj = b.y, zj = b.z;
  if (img) {
    xj = xadd(xj, (double)ix * g.box);
    yj = xadd(yj, (double)iy * g.box);
    zj = xadd(zj, (double)iz * g.box);
  }
  return norm2_exact(xsub(a.x, xj), xsub(a.y, yj), xsub(a.z, zj)) < rcutsq;
}

// One atom of the FP32 LJ force: the compact row, or (skin tripped) the full
// candidate row with a refresh of the compact row.  ev: E, E_shifted, W.
template <bool ENERGY>
__device__ __forceinline__ void lj32_atom(int i, const float4* __restrict__ posf,
                                          const md_double4* __restrict__ pos,
                                          double* __restrict__ f3, int ld,
                                          uint32_t* __restrict__ list, int* __restrict__ len,
                                          const RowWalker& w, bool tripped, int* skin, int cap,
                                          float rv2, float4* __restrict__ pos_build,
                                          double rcutsq, const Species& sp, double* ev) {
  const float4 pi = posf[i];
  const int ti = __float_as_int(pi.w);
  const float rc2 = (float)rcutsq;
  const float rc_lo = rc2 * (1.0f - 1e-5f), rc_hi = rc2 * (1.0f + 1e-5f);
  const float Lf = w.g.box_f, Llo = w.g.box_lo;
  float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
  float cx = 0.f, cy = 0.f, cz = 0.f;
  int inchunk = 0;
  auto visit = [&](int j, int ix, int iy, int iz, bool img) {
    const float4 pj = posf[j];
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    if (img) {
      dx = (pi.x - fmaf((float)ix, Lf, pj.x)) - (float)ix * Llo;
      dy = (pi.y - fmaf((float)iy, Lf, pj.y)) - (float)iy * Llo;
      dz = (pi.z - fmaf((float)iz, Lf, pj.z)) - (float)iz * Llo;
    }
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (!lj_inside(r2, rc_lo, rc_hi, pos, i, j, img, ix, iy, iz, w.g, rcutsq)) return;
    const int tj = __float_as_int(pj.w);
    if (tj != SP_NG && ti != SP_NG) return;
    const int sel = lj_select(ti, tj);
    const float sig = sp.sig[sel], eps = sp.eps[sel];
    const float inv = 1.0f / r2;
    const float sr2 = sig * sig * inv;
    const float sr6 = sr2 * sr2 * sr2;
    const float fij = (24.0f * eps) * inv * sr6 * (2.0f * sr6 - 1.0f);
    cx = fmaf(dx, fij, cx);
    cy = fmaf(dy, fij, cy);
    cz = fmaf(dz, fij, cz);
    if (ENERGY) {
      const float src2 = sig * sig / rc2;
      const float src6 = src2 * src2 * src2;
      const float e = 2.0f * eps * (sr6 * sr6 - sr6);
      ev[0] += (double)e;
      ev[1] += (double)e - (double)(2.0f * eps * (src6 * src6 - src6));
      ev[2] += 0.5 * (double)(r2 * fij);
    }
    if (++inchunk == 16) {
      kahan(hx, lx, cx);
      kahan(hy, ly, cy);
      kahan(hz, lz, cz);
      cx = cy = cz = 0.f;
      inchunk = 0;
    }
  };
  if (!tripped) {
    const int L = len[i];
    for (int k = 0; k < L; k++) {
      const uint32_t e = list[(size_t)k * ld + i];
      visit(entry_index(e), entry_img(e, 0), entry_img(e, 1), entry_img(e, 2), (e >> 26) != 0);
    }
  } else {
    // skin exceeded: walk the full candidate row (the reference's row, same
    // order) and refresh this atom's compact row at the current positions
    const float4 pc = pi;
    int kept = 0;
    walk_row(w, pos, i, [&](int m, int ix, int iy, int iz) {
      visit(m, ix, iy, iz, w.g.periodic && (ix | iy | iz));
      const float4 pm = posf[m];
      const float dx = pc.x - (pm.x + (float)ix * w.g.box_f);
      const float dy = pc.y - (pm.y + (float)iy * w.g.box_f);
      const float dz = pc.z - (pm.z + (float)iz * w.g.box_f);
      if (dx * dx + dy * dy + dz * dz < rv2) {
        if (kept < cap) list[(size_t)kept * ld + i] = pack_entry(m, ix, iy, iz);
        kept++;
      }
    });
    if (kept > cap) atomicOr(&skin[2], 1);
    len[i] = kept < cap ? kept : cap;
    pos_build[i] = pc;
  }
  kahan(hx, lx, cx);
  kahan(hy, ly, cy);
  kahan(hz, lz, cz);
  f3[3 * i] = (double)hx - (double)lx;
  f3[3 * i + 1] = (double)hy - (double)ly;
  f3[3 * i + 2] = (double)hz - (double)lz;
}

// out-of-line copy of the tripped path for the TMA kernel (keeps its
// register allocation free of the rarely used full-row walk)
__device__ __noinline__ void lj32_atom_tripped(int i, const float4* posf, const md_double4* pos,
                                              double* f3, int ld, uint32_t* list, int* len,
                                              const RowWalker& w, int* skin, int cap, float rv2,
                                              float4* pos_build, double rcutsq,
                                              const Species& sp) {
  double ev[3];
  lj32_atom<false>(i, posf, pos, f3, ld, list, len, w, true, skin, cap, rv2, pos_build, rcutsq,
                   sp, ev);
}

template <bool ENERGY>
__global__ void __launch_bounds__(128)
    k_lj_fp32(const float4* __restrict__ posf, const md_double4* __restrict__ pos,
              double* __restrict__ f3, int n, int ld, uint32_t* __restrict__ list,
              int* __restrict__ len, RowWalker w, int* skin, int parity, int cap, float rv2,
              float4* __restrict__ pos_build, double rcutsq, Species sp,
              double* __restrict__ epart) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ev[3] = {0.0, 0.0, 0.0};
  const bool tripped = (skin[parity] | skin[2]) != 0;
  if (i < n)
    lj32_atom<ENERGY>(i, posf, pos, f3, ld, list, len, w, tripped, skin, cap, rv2, pos_build,
                      rcutsq, sp, ev);
  if (tripped && i == 0) atomicAdd(&skin[3], 1);
  if (i == 0) skin[parity ^ 1] = 0;  // the next step's flag starts clear
  if (ENERGY) block_partial<3>(ev, epart);
}

// The FP32 LJ force with the compact list streamed through shared memory by
// TMA: each block of 128 atoms walks its list in tiles of 16 slots x 128
// atoms (8 KB), double-buffered and synchronised with mbarriers, so that
// list traffic is bulk and in flight while the pairs of the previous tile
// are computed.  Positions are gathered through L1.  Each tile's FP32 sums
// are folded into a compensated (Kahan) FP32 pair.  ALL_NG: every atom is of
// the NG species (one parameter set, no type tests).
template <bool ALL_NG>
__global__ void __launch_bounds__(kListTileAtoms, 8)
    k_lj_tma(const __grid_constant__ CUtensorMap tmap, const float4* __restrict__ posf,
             const md_double4* __restrict__ pos, double* __restrict__ f3, int n, int ld,
             uint32_t* __restrict__ list, int* __restrict__ len, RowWalker w, int* skin,
             int parity, int cap, float rv2, float4* __restrict__ pos_build, double rcutsq,
             Species sp, int* status, int wait_limit) {
  __shared__ __align__(128) uint32_t tile[2][kListTileSlots][kListTileAtoms];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int s_max[kListTileAtoms / 32];
  const int tid = threadIdx.x;
  const int i = blockIdx.x * kListTileAtoms + tid;
  const bool tripped = (skin[parity] | skin[2]) != 0;
  if (tripped) {
    if (i < n)
      lj32_atom_tripped(i, posf, pos, f3, ld, list, len, w, skin, cap, rv2, pos_build, rcutsq,
                        sp);
    if (i == 0) {
      atomicAdd(&skin[3], 1);
      skin[parity ^ 1] = 0;
    }
    return;
  }
  const int L = i < n ? len[i] : 0;
  int m = L;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((tid & 31) == 0) s_max[tid >> 5] = m;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  int maxlen = s_max[0];
#pragma unroll
  for (int k = 1; k < kListTileAtoms / 32; k++) maxlen = max(maxlen, s_max[k]);
  const int T = (maxlen + kListTileSlots - 1) / kListTileSlots;
  constexpr uint32_t kTileBytes = kListTileSlots * kListTileAtoms * 4;
  const int x0 = blockIdx.x * kListTileAtoms;
  if (tid == 0) {
    for (int t = 0; t < 2 && t < T; t++) {
      mbar_expect_tx(&bar[t], kTileBytes);
      tma_load_2d(&tile[t][0][0], &tmap, x0, t * kListTileSlots, &bar[t]);
    }
  }
  const float4 pi = i < n ? posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int ti = __float_as_int(pi.w);
  const float rc2 = (float)rcutsq;
  const float rc_lo = rc2 * (1.0f - 1e-5f), rc_hi = rc2 * (1.0f + 1e-5f);
  const float Lf = w.g.box_f, Llo = w.g.box_lo;
  // NG-NG parameters, and the two cross parameter sets for mixed systems
  const float s2_ng = sp.sig[2] * sp.sig[2], c_ng = 24.0f * sp.eps[2];
  const float s2_n = sp.sig[0] * sp.sig[0], c_n = 24.0f * sp.eps[0];
  const float s2_o = sp.sig[1] * sp.sig[1], c_o = 24.0f * sp.eps[1];
  float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
  bool ok = true;
  int failed_at = 0;
  for (int t = 0; t < T; t++) {
    const int b = t & 1;
    // the outcome is made block-uniform, so every thread leaves together
    if (!__syncthreads_and(mbar_wait(&bar[b], (uint32_t)((t >> 1) & 1), status, wait_limit))) {
      ok = false;
      failed_at = t;
      break;
    }
    const int kmax = min(kListTileSlots, L - t * kListTileSlots);
    float cx = 0.f, cy = 0.f, cz = 0.f;
    // every slot is evaluated by every lane (no divergence); slots past the
    // atom's row read the atom itself and contribute zero
#pragma unroll 4
    for (int kk = 0; kk < kListTileSlots; kk++) {
      const bool valid = kk < kmax;
      const uint32_t e = valid ? tile[b][kk][tid] : (uint32_t)(i < n ? i : 0);
      const int j = entry_index(e);
      const float4 pj = __ldg(&posf[j]);
      float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
      if (e >> 26) {  // periodic image (rare: boundary cells only)
        const float fx = (float)entry_img(e, 0), fy = (float)entry_img(e, 1),
                    fz = (float)entry_img(e, 2);
        dx = (pi.x - fmaf(fx, Lf, pj.x)) - fx * Llo;
        dy = (pi.y - fmaf(fy, Lf, pj.y)) - fy * Llo;
        dz = (pi.z - fmaf(fz, Lf, pj.z)) - fz * Llo;
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
      const float sr6 = sr2 * sr2 * sr2;
      float fij = c24 * inv * sr6 * fmaf(2.0f, sr6, -1.0f);
      bool in = r2 <= rc_lo;
      if (use && !in && r2 < rc_hi)  // within 1e-5 of the cutoff: decide in FP64
        in = lj_inside(r2, rc_lo, rc_hi, pos, i, j, (e >> 26) != 0, entry_img(e, 0),
                       entry_img(e, 1), entry_img(e, 2), w.g, rcutsq);
      fij = (use && in) ? fij : 0.0f;
      cx = fmaf(dx, fij, cx);
      cy = fmaf(dy, fij, cy);
      cz = fmaf(dz, fij, cz);
    }
    kahan(hx, lx, cx);
    kahan(hy, ly, cy);
    kahan(hz, lz, cz);
    __syncthreads();  // everyone is done with buffer b
    if (tid == 0 && t + 2 < T) {
      fence_proxy_async();
      mbar_expect_tx(&bar[b], kTileBytes);
      tma_load_2d(&tile[b][0][0], &tmap, x0, (t + 2) * kListTileSlots, &bar[b]);
    }
  }
  if (!ok) {
    // tiles failed_at and failed_at + 1 may still be in flight: they land in
    // this block's shared memory before it leaves
    if (tid == 0)
      for (int t = failed_at; t < failed_at + 2 && t < T; t++)
        mbar_drain(&bar[t & 1], (uint32_t)((t >> 1) & 1), status);
    return;
  }
  if (i < n) {
    f3[3 * i] = (double)hx - (double)lx;
    f3[3 * i + 1] = (double)hy - (double)ly;
    f3[3 * i + 2] = (double)hz - (double)lz;
  }
  if (i == 0) skin[parity ^ 1] = 0;  // the next step's flag starts clear
}

// --------------------------------------------------------------- bond order
template <typename T>
struct PosT;
template <>
struct PosT<double> {
  static __device__ __forceinline__ void load(const md_double4* pos, const float4*, int j,
                                              double& x, double& y, double& z, int& t) {
    md_double4 p = pos[j];
    x = p.x;
    y = p.y;
    z = p.z;
    t = (int)p.w;
  }
  // image position: p + img * L, exactly as the oracle forms it
  static __device__ __forceinline__ void image(double& x, double& y, double& z, uint32_t e,
                                               const Grid& g) {
    if (e >> 26) image3(x, y, z, entry_img(e, 0), entry_img(e, 1), entry_img(e, 2), g);
  }
  static __device__ __forceinline__ void image3(double& x, double& y, double& z, int ix,
                                                int iy, int iz, const Grid& g) {
    x = xadd(x, (double)ix * g.box);
    y = xadd(y, (double)iy * g.box);
    z = xadd(z, (double)iz * g.box);
  }
};
template <>
struct PosT<float> {
  static __device__ __forceinline__ void load(const md_double4*, const float4* posf, int j,
                                              float& x, float& y, float& z, int& t) {
    float4 p = posf[j];
    x = p.x;
    y = p.y;
    z = p.z;
    t = __float_as_int(p.w);
  }
  static __device__ __forceinline__ void image(float& x, float& y, float& z, uint32_t e,
                                               const Grid& g) {
    if (e >> 26) image3(x, y, z, entry_img(e, 0), entry_img(e, 1), entry_img(e, 2), g);
  }
  static __device__ __forceinline__ void image3(float& x, float& y, float& z, int ix, int iy,
                                                int iz, const Grid& g) {
    x = fmaf((float)ix, g.box_f, x) + (float)ix * g.box_lo;
    y = fmaf((float)iy, g.box_f, y) + (float)iy * g.box_lo;
    z = fmaf((float)iz, g.box_f, z) + (float)iz * g.box_lo;
  }
};

// short list: candidates within rcut at the current positions, row order
template <typename T>
__global__ void __launch_bounds__(128)
    k_mb_short(const md_double4* __restrict__ pos, const float4* __restrict__ posf, int n,
               int ld, const uint32_t* __restrict__ list, const int* __restrict__ len, Grid g,
               double rcutsq, uint32_t* __restrict__ sl, int* __restrict__ slen,
               const int* __restrict__ run_if) {
  if (run_if && *run_if == 0) return;  // the whole launch: a gated call with nothing to do
  // one warp per atom, lanes over its row: the kept entries in row order
  // (ballot prefix), 32 candidates tested at a time
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;  // whole warp
  T xi, yi, zi;
  int ti;
  PosT<T>::load(pos, posf, i, xi, yi, zi, ti);
  const T rc2 = (T)rcutsq;
  const T band = (T)1e-5 * rc2;
  int cnt = 0;
  const int L = len[i];
  for (int k0 = 0; k0 < L; k0 += 32) {
    const int k = k0 + lane;
    bool keep = false;
    uint32_t e = 0;
    if (k < L) {
      e = list[(size_t)k * ld + i];
      const int j = entry_index(e);
      T xj, yj, zj;
      int tj;
      PosT<T>::load(pos, posf, j, xj, yj, zj, tj);
      PosT<T>::image(xj, yj, zj, e, g);
      T r2;
      if (sizeof(T) == 8)
        r2 = (T)norm2_exact((double)(xi - xj), (double)(yi - yj), (double)(zi - zj));
      else
        r2 = (xi - xj) * (xi - xj) + (yi - yj) * (yi - yj) + (zi - zj) * (zi - zj);
      keep = r2 < rc2;
      if (sizeof(T) == 4 && r2 > rc2 - band && r2 < rc2 + band) {
        double a[3], b[3];
        int t0;
        PosT<double>::load(pos, posf, i, a[0], a[1], a[2], t0);
        PosT<double>::load(pos, posf, j, b[0], b[1], b[2], t0);
        PosT<double>::image(b[0], b[1], b[2], e, g);
        keep = norm2_exact(xsub(a[0], b[0]), xsub(a[1], b[1]), xsub(a[2], b[2])) < rcutsq;
      }
    }
    const unsigned mask = __ballot_sync(0xffffffffu, keep);
    if (keep) sl[(size_t)(cnt + __popc(mask & ((1u << lane) - 1u))) * n + i] = e;
    cnt += __popc(mask);
  }
  if (lane == 0) slen[i] = cnt;
}

// Third bodies m of the warp's atom i (pass 1): what depends on i and m
// only, computed once per warp instead of once per pair i-j.  In FP64 with
// the expressions of the per-pair evaluation, so the values are the same.
constexpr int kThirdMax = 64;
template <typename T>
struct ThirdSm {
  T x[kThirdMax], y[kThirdMax], z[kThirdMax];  // position at its image
  T r[kThirdMax], ir[kThirdMax], fc[kThirdMax], dfc[kThirdMax];  // r_im, 1 / r_im (FP32)
  T ux[kThirdMax], uy[kThirdMax], uz[kThirdMax];                // (r_i - r_m) / r_im
  int id[kThirdMax];                                            // atom, -1 for an NG atom
};

// FP32: 64 registers without spills, 8 blocks per SM instead of 7 (FP64
// instances keep their registers: a bound there spills)
template <typename T, bool ENERGY>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 0)
    k_mb_pass1(const md_double4* __restrict__ pos, const float4* __restrict__ posf,
               double* __restrict__ f3, int n, const uint32_t* __restrict__ sl,
               const int* __restrict__ slen, Grid g, int ljexist, T* __restrict__ xsi_s,
               T* __restrict__ xsj_s, double* __restrict__ epart,
               double* __restrict__ eatom, const int* __restrict__ run_if) {
  if (!ENERGY && run_if && *run_if == 0) return;
  const int warps = blockDim.x >> 5;
  const int i = blockIdx.x * warps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  // FP32: hardware rsqrt for distances and their reciprocals, and the
  // third bodies' terms staged in FP32 (FP64: exact roots and quotients)
  constexpr bool kFast = std::is_same<T, float>::value;
  double ev[2] = {0.0, 0.0};
  __shared__ ThirdSm<T> third_sm[4];
  ThirdSm<T>& TS = third_sm[(threadIdx.x >> 5) & 3];
  if (i < n) {
    T xi, yi, zi;
    int ti;
    PosT<T>::load(pos, posf, i, xi, yi, zi, ti);
    const int S = slen[i];
    T fx = 0, fy = 0, fz = 0;
    const T cut_rijsq = (T)MD_CUTOFF_RIJSQ;
    const T nanv = (T)NAN;
    const bool staged = S <= kThirdMax && blockDim.x <= 128;  // warp-uniform
    if (staged) {
      for (int m = lane; m < S; m += 32) {
        const uint32_t em = sl[(size_t)m * n + i];
        const int mp = entry_index(em);
        T xm, ym, zm;
        int tm;
        PosT<T>::load(pos, posf, mp, xm, ym, zm, tm);
        PosT<T>::image(xm, ym, zm, em, g);
        TS.id[m] = tm == SP_NG ? -1 : mp;
        TS.x[m] = xm;
        TS.y[m] = ym;
        TS.z[m] = zm;
        if constexpr (kFast) {
          const float imx = xi - xm, imy = yi - ym, imz = zi - zm;
          const float r2 = imx * imx + imy * imy + imz * imz;
          const float irim = rsqrtf(r2), rim = r2 * irim;
          float fci, dfci;
          cutoff<float>(rim, fci, dfci);
          TS.r[m] = rim;
          TS.ir[m] = irim;
          TS.fc[m] = fci;
          TS.dfc[m] = dfci;
          TS.ux[m] = imx * irim;
          TS.uy[m] = imy * irim;
          TS.uz[m] = imz * irim;
        } else {
          // the per-pair branch's expressions below, once per third body
          const T imx = xi - xm, imy = yi - ym, imz = zi - zm;
          const T rim = md_sqrt(imx * imx + imy * imy + imz * imz);
          T fci, dfci;
          cutoff<T>(rim, fci, dfci);
          TS.r[m] = rim;
          TS.ir[m] = fdiv<T>(1.0, rim);
          TS.fc[m] = fci;
          TS.dfc[m] = dfci;
          TS.ux[m] = fdiv<T>(imx, rim);
          TS.uy[m] = fdiv<T>(imy, rim);
          TS.uz[m] = fdiv<T>(imz, rim);
        }
      }
      __syncwarp();
    }
    for (int s = lane; s < S; s += 32) {
      const uint32_t e = sl[(size_t)s * n + i];
      const int j = entry_index(e);
      T xj, yj, zj;
      int tj;
      PosT<T>::load(pos, posf, j, xj, yj, zj, tj);
      PosT<T>::image(xj, yj, zj, e, g);
      const size_t slot = (size_t)s * n + i;
      const T ijx = xi - xj, ijy = yi - yj, ijz = zi - zj;
      T rij = ijx * ijx + ijy * ijy + ijz * ijz;
      if (tj == SP_NG || rij > cut_rijsq) {
        xsi_s[slot] = nanv;
        xsj_s[slot] = nanv;
        continue;
      }
      rij = md_sqrt(rij);
      // BondOrderFuncs.h:242-278 bondForces
      T va = 0, dva = 0, vr = 0, dvr = 0, vdw, dvdw, bo = 0;
      T dbx = 0, dby = 0, dbz = 0;
      T fcut, dfcut;
      cutoff<T>(fdiv<T>(rij, 10), fcut, dfcut);
      T xs_i = nanv, xs_j = nanv;
      if (fcut > 0) {
        const T de = get_de<T>(ti, tj), re = get_re<T>(ti, tj), beta = get_beta<T>(ti, tj);
        attractive<T>(va, dva, rij, de, beta, re);
        repulsive<T>(vr, dvr, rij, de, beta, re);
        // BondOrderFuncs.h:12-143 bondOrder1
        const T drijx = fdiv<T>(ijx, rij), drijy = fdiv<T>(ijy, rij), drijz = fdiv<T>(ijz, rij);
        const T E = md_exp((T)MD_LAMDA3 * (rij - re));
        const T inv_rij = fdiv<T>(1.0f, rij), half_inv_rij = 0.5f * inv_rij;
        T xsi = 0, xsj = 0;
        T dxsix = 0, dxsiy = 0, dxsiz = 0, dxsjx = 0, dxsjy = 0, dxsjz = 0;
        for (int m = 0; m < S; m++) {
          T xm, ym, zm, rim, inv_rim, fci, dfci, drimx, drimy, drimz;
          if (staged) {
            const int mp = TS.id[m];
            if (mp < 0 || mp == j) continue;
            xm = TS.x[m];
            ym = TS.y[m];
            zm = TS.z[m];
            rim = TS.r[m];
            inv_rim = TS.ir[m];
            fci = TS.fc[m];
            dfci = TS.dfc[m];
            drimx = TS.ux[m];
            drimy = TS.uy[m];
            drimz = TS.uz[m];
          } else {
            const uint32_t em = sl[(size_t)m * n + i];
            const int mp = entry_index(em);
            int tm;
            PosT<T>::load(pos, posf, mp, xm, ym, zm, tm);
            if (tm == SP_NG || mp == j) continue;
            PosT<T>::image(xm, ym, zm, em, g);
            const T imx = xi - xm, imy = yi - ym, imz = zi - zm;
            rim = md_sqrt(imx * imx + imy * imy + imz * imz);
            cutoff<T>(rim, fci, dfci);
            drimx = fdiv<T>(imx, rim);
            drimy = fdiv<T>(imy, rim);
            drimz = fdiv<T>(imz, rim);
            inv_rim = fdiv<T>(1.0f, rim);
          }
          const T jmx = xj - xm, jmy = yj - ym, jmz = zj - zm;
          T rjm, inv_rjm = 0;
          if constexpr (kFast) {  // the distance and its reciprocal from one rsqrt
            const float r2 = (float)(jmx * jmx + jmy * jmy + jmz * jmz);
            const float ir = rsqrtf(r2);
            inv_rjm = ir;
            rjm = r2 * ir;
          } else {
            rjm = md_sqrt(jmx * jmx + jmy * jmy + jmz * jmz);
            inv_rjm = fdiv<T>(1.0, rjm);
          }
          T fcj, dfcj;
          cutoff<T>(rjm, fcj, dfcj);
          if (fci > 0) {
            // d cos / d r_i = drij (1/rim - cos/rij) + drim (1/rij - cos/rim): the
            // reference's quotient per component (BondOrderFuncs.h) in two scalars
            const T num2 = rij * rij + rim * rim - rjm * rjm;
            const T icos = num2 * half_inv_rij * inv_rim;
            T gth, gpre;
            angular1<T>(icos, gth, gpre);
            xsi += fci * gth * E;
            const T fE = fci * E;
            const T cm = dfci * gth * E + fE * gpre * (inv_rij - icos * inv_rim);
            const T cj = fE * (gpre * (inv_rim - icos * inv_rij) + gth * (T)MD_LAMDA3);
            dxsix = fma(drimx, cm, fma(drijx, cj, dxsix));
            dxsiy = fma(drimy, cm, fma(drijy, cj, dxsiy));
            dxsiz = fma(drimz, cm, fma(drijz, cj, dxsiz));
          }
          if (fcj > 0) {
            // d cos / d r_i = drij (1/rjm - cos/rij) - drim rim / (rij rjm)
            const T num2 = rij * rij + rjm * rjm - rim * rim;
            const T jcos = num2 * half_inv_rij * inv_rjm;
            T gth, gpre;
            angular1<T>(jcos, gth, gpre);
            xsj += fcj * gth * E;
            const T fE = fcj * E;
            const T cj = fE * (gpre * (inv_rjm - jcos * inv_rij) + (T)MD_LAMDA3 * gth);
            const T cm = -fE * gpre * rim * inv_rij * inv_rjm;
            dxsjx = fma(drijx, cj, fma(drimx, cm, dxsjx));
            dxsjy = fma(drijy, cj, fma(drimy, cm, dxsjy));
            dxsjz = fma(drijz, cj, fma(drimz, cm, dxsjz));
          }
        }
        xs_i = xsi;
        xs_j = xsj;
        const T bij = fdiv<T>(1.0f, 1.0f + xsi), pbi = fdiv<T>(1.0f, (1.0f + xsi) * (1.0f + xsi));
        const T bji = fdiv<T>(1.0f, 1.0f + xsj), pbj = fdiv<T>(1.0f, (1.0f + xsj) * (1.0f + xsj));
        bo = 0.5f * (bij + bji);
        dbx = 0.5f * (pbi * dxsix + pbj * dxsjx);
        dby = 0.5f * (pbi * dxsiy + pbj * dxsjy);
        dbz = 0.5f * (pbi * dxsiz + pbj * dxsjz);
        // what pass 2 needs of this pair: va E / (4 (1 + xi)^2) for either
        // end (its force is -factor x the derivative of the angle terms)
        xs_i = (T)0.25 * va * E * pbi;
        xs_j = (T)0.25 * va * E * pbj;
      }
      xsi_s[slot] = xs_i;
      xsj_s[slot] = xs_j;
      vander_waals<T>(vdw, dvdw, rij, get_r0v<T>(ti, tj));
      const T fij = dvr - bo * dva + dvdw;
      fx += fdiv<T>(fij * ijx, rij) - dbx * va;
      fy += fdiv<T>(fij * ijy, rij) - dby * va;
      fz += fdiv<T>(fij * ijz, rij) - dbz * va;
      if (ENERGY) ev[0] += (double)(0.5f * ((vr - bo * va) + vdw));
    }
    double sx = warp_sum((double)fx), sy = warp_sum((double)fy), sz = warp_sum((double)fz);
    if (ENERGY && eatom) {
      // per-atom share: sum over j of 1/2 (Vr - b Va + Vdw) (the i-sum of
      // common/DebugCalculations.cpp:129-270 restricted to the force's pairs)
      const double ei = warp_sum(ev[0]);
      if (lane == 0) eatom[i] = ei;
    }
    if (lane == 0) {
      if (ljexist) {
        f3[3 * i] += sx;
        f3[3 * i + 1] += sy;
        f3[3 * i + 2] += sz;
      } else {
        f3[3 * i] = sx;
        f3[3 * i + 1] = sy;
        f3[3 * i + 2] = sz;
      }
      if (ENERGY) {
        const md_double4 p = pos[i];
        ev[1] = p.x * sx + p.y * sy + p.z * sz;
      }
    }
  }
  if (ENERGY) block_partial<2>(ev, epart);
}

// the part of pass 2 for one pair (i, j) of the warp's atom k: i at (x, y, z)
// with its k-side terms, j = entry sl[q]; adds -F_k to (fx, fy, fz)
template <typename T>
struct Pass2I {
  T x, y, z, r, ir, fc, dfc, ux, uy, uz;
  int id;
};

// r and 1/r from r^2: one rsqrt in FP32; the square root and a quotient in FP64
template <typename T>
__device__ __forceinline__ void dist_recip(T r2, T& r, T& ir) {
  if constexpr (std::is_same<T, float>::value) {
    ir = rsqrtf(r2);
    r = r2 * ir;
  } else {
    r = md_sqrt(r2);
    ir = fdiv<T>(1.0, r);
  }
}

template <typename T>
__device__ __forceinline__ void pass2_pair(const Pass2I<T>& I, size_t q, int k, T xk, T yk, T zk,
                                           const md_double4* pos, const float4* posf,
                                           const uint32_t* sl, const Grid& g, const int* cell3,
                                           const int* ref_rows, int ref_nls, int ref_nlargest,
                                           T rc2, T cut_rijsq, const T* wi_s, const T* wj_s,
                                           T& fx, T& fy, T& fz, int& miss) {
  const int jp = entry_index(sl[q]);
  if (jp == k) return;
  int im[3] = {0, 0, 0};
  if (ref_rows) {
    // caller-supplied rows (no periodic box): is jp in row k?
    const int* row = ref_rows + (size_t)k * ref_nls;
    bool found = false;
    for (int q2 = 0; q2 < ref_nlargest && row[q2] != -1; q2++)
      if (row[q2] == jp) {
        found = true;
        break;
      }
    if (!found) return;
  } else if (!in_row(cell3, g, k, jp, im)) {
    return;
  }
  // j at its image in k's row, as BondOrderFuncs.h:367-369 sees it
  T xj, yj, zj;
  int tj;
  PosT<T>::load(pos, posf, jp, xj, yj, zj, tj);
  if (im[0] | im[1] | im[2]) PosT<T>::image3(xj, yj, zj, im[0], im[1], im[2], g);
  const T ijx = I.x - xj, ijy = I.y - yj, ijz = I.z - zj;
  const T r2ij = ijx * ijx + ijy * ijy + ijz * ijz;
  if (r2ij >= rc2 || r2ij > cut_rijsq) return;
  const T wi = wi_s[q], wj = wj_s[q];
  if (wi != wi || tj == SP_NG) {
    miss++;
    return;
  }
  T rij, irij, rjk, irjk;
  dist_recip<T>(r2ij, rij, irij);
  const T half_irij = (T)0.5 * irij;
  const T jkx = xj - xk, jky = yj - yk, jkz = zj - zk;
  dist_recip<T>(jkx * jkx + jky * jky + jkz * jkz, rjk, irjk);
  const T drjkx = -jkx * irjk, drjky = -jky * irjk, drjkz = -jkz * irjk;
  T fcj, dfcj;
  cutoff<T>(rjk, fcj, dfcj);
  T ck = 0, cj = 0;  // coefficients of d_ik and d_jk in -F_k
  if (I.fc > 0) {
    // d cos / d r_k = drik (1/rij - cos/rik) - drjk rjk / (rij rik)
    const T icos = (rij * rij + I.r * I.r - rjk * rjk) * half_irij * I.ir;
    T gth, gpre;
    angular1<T>(icos, gth, gpre);
    ck = wi * (I.dfc * gth + I.fc * gpre * (irij - icos * I.ir));
    cj = -wi * I.fc * gpre * rjk * irij * I.ir;
  }
  if (fcj > 0) {
    // d cos / d r_k = drjk (1/rij - cos/rjk) - drik rik / (rij rjk)
    const T jcos = (rij * rij + rjk * rjk - I.r * I.r) * half_irij * irjk;
    T gth, gpre;
    angular1<T>(jcos, gth, gpre);
    cj = fma(wj, dfcj * gth + fcj * gpre * (irij - jcos * irjk), cj);
    ck = fma(-wj * fcj * gpre, I.r * irij * irjk, ck);
  }
  fx -= fma(I.ux, ck, drjkx * cj);
  fy -= fma(I.uy, ck, drjky * cj);
  fz -= fma(I.uz, ck, drjkz * cj);
}

template <typename T>
__device__ __forceinline__ Pass2I<T> pass2_entry(uint32_t ei, T xk, T yk, T zk,
                                                 const md_double4* pos, const float4* posf,
                                                 const Grid& g) {
  Pass2I<T> I;
  I.id = entry_index(ei);
  int ti;
  PosT<T>::load(pos, posf, I.id, I.x, I.y, I.z, ti);
  PosT<T>::image(I.x, I.y, I.z, ei, g);
  const T ikx = xk - I.x, iky = yk - I.y, ikz = zk - I.z;
  dist_recip<T>(ikx * ikx + iky * iky + ikz * ikz, I.r, I.ir);
  cutoff<T>(I.r, I.fc, I.dfc);
  I.ux = ikx * I.ir;
  I.uy = iky * I.ir;
  I.uz = ikz * I.ir;
  return I;
}

// Pass 2 (BondOrderFuncs.h:148-237 bondOrder2 for every pair i-j with k as
// third body), one entry i of k's short list per lane.  Per pair, pass 1
// left va E / (4 (1 + xi_ij)^2) and va E / (4 (1 + xi_ji)^2) in the slot, so
// the exponential and the two quotients of the reference's per-triplet
// expression are not evaluated again here; NaN marks a slot pass 1 did not
// evaluate (its va is 0: counted as missing, no force).  Each angle's
// derivative takes the shorter equal form (test_bond_order_identities: equal
// to 1e-13 in FP64) with one reciprocal per distance: one rsqrt in FP32, a
// square root and a quotient in FP64.  (Spreading the (i, j) pairs of k over
// all 32 lanes through a prefix of the row lengths was measured slower in
// FP32, 348 against 249 us on 32,768 atoms: lanes of one i read 32 different
// lines of the slot arrays, where lanes of neighbouring i, stored side by
// side, share sectors.)
// FP32: 40 registers, 12 blocks per SM instead of 10 (FP64 instances keep
// their registers)
template <typename T, bool ENERGY>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 12 : 0)
    k_mb_pass2(const md_double4* __restrict__ pos, const float4* __restrict__ posf,
               double* __restrict__ f3, int n, const uint32_t* __restrict__ sl,
               const int* __restrict__ slen, Grid g, const int* __restrict__ cell3,
               const int* __restrict__ ref_rows, int ref_nls, int ref_nlargest, double rcutsq,
               const T* __restrict__ wi_s, const T* __restrict__ wj_s,
               int* __restrict__ missing, double* __restrict__ epart,
               const int* __restrict__ run_if) {
  if (!ENERGY && run_if && *run_if == 0) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * 4 + warp;
  double ev[1] = {0.0};
  if (k < n) {
    T xk, yk, zk;
    int tk;
    PosT<T>::load(pos, posf, k, xk, yk, zk, tk);
    const int Sk = slen[k];
    const T rc2 = (T)rcutsq, cut_rijsq = (T)MD_CUTOFF_RIJSQ;
    T fx = 0, fy = 0, fz = 0;
    int miss = 0;
    for (int s = lane; s < Sk; s += 32) {
      const Pass2I<T> I = pass2_entry<T>(sl[(size_t)s * n + k], xk, yk, zk, pos, posf, g);
      const int Si = slen[I.id];
      for (int sj = 0; sj < Si; sj++)
        pass2_pair<T>(I, (size_t)sj * n + I.id, k, xk, yk, zk, pos, posf, sl, g, cell3,
                      ref_rows, ref_nls, ref_nlargest, rc2, cut_rijsq, wi_s, wj_s, fx, fy, fz,
                      miss);
    }
    const double sx = warp_sum((double)fx), sy = warp_sum((double)fy), sz = warp_sum((double)fz);
    const int m = __reduce_add_sync(0xffffffffu, miss);
    if (lane == 0) {
      f3[3 * k] += sx;
      f3[3 * k + 1] += sy;
      f3[3 * k + 2] += sz;
      if (m) atomicAdd(missing, m);
      if (ENERGY) {
        const md_double4 p = pos[k];
        ev[0] = p.x * sx + p.y * sy + p.z * sz;
      }
    }
  }
  if (ENERGY) block_partial<1>(ev, epart);
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

void launch_lj(const ForceArgs& a, bool fp32, bool energy, cudaStream_t st) {
  const int T = 128;
  const int B = nblk(a.n, T);
  if (B == 0) return;
  if (!fp32) {
    if (energy)
      k_lj_fp64<true><<<B, T, 0, st>>>(a.pos, a.f3, a.n, a.ld, a.list, a.len, a.walker, a.skin,
                                       a.parity, a.cap, a.rv2, a.pos_build, a.rcutsq, a.sp,
                                       a.epart);
    else
      k_lj_fp64<false><<<B, T, 0, st>>>(a.pos, a.f3, a.n, a.ld, a.list, a.len, a.walker, a.skin,
                                        a.parity, a.cap, a.rv2, a.pos_build, a.rcutsq, a.sp,
                                        a.epart);
  } else if (!energy && a.tmap) {
    const int TB = nblk(a.n, kListTileAtoms);
    if (a.all_ng)
      k_lj_tma<true><<<TB, kListTileAtoms, 0, st>>>(*a.tmap, a.posf, a.pos, a.f3, a.n, a.ld,
                                                    a.list, a.len, a.walker, a.skin, a.parity,
                                                    a.cap, a.rv2, a.pos_build, a.rcutsq, a.sp,
                                                    a.status, a.wait_limit);
    else
      k_lj_tma<false><<<TB, kListTileAtoms, 0, st>>>(*a.tmap, a.posf, a.pos, a.f3, a.n, a.ld,
                                                     a.list, a.len, a.walker, a.skin, a.parity,
                                                     a.cap, a.rv2, a.pos_build, a.rcutsq, a.sp,
                                                     a.status, a.wait_limit);
  } else {
    if (energy)
      k_lj_fp32<true><<<B, T, 0, st>>>(a.posf, a.pos, a.f3, a.n, a.ld, a.list, a.len, a.walker,
                                       a.skin, a.parity, a.cap, a.rv2, a.pos_build, a.rcutsq,
                                       a.sp, a.epart);
    else
      k_lj_fp32<false><<<B, T, 0, st>>>(a.posf, a.pos, a.f3, a.n, a.ld, a.list, a.len, a.walker,
                                        a.skin, a.parity, a.cap, a.rv2, a.pos_build, a.rcutsq,
                                        a.sp, a.epart);
  }
}

int lj_blocks(int n) { return nblk(n, 128); }
int mb_blocks(int n) { return nblk(n, 4); }

template <typename T, bool ENERGY>
static void launch_pass2(const MbArgs& a, int B, T* xsi, T* xsj, cudaStream_t st) {
  k_mb_pass2<T, ENERGY><<<B, 128, 0, st>>>(a.pos, a.posf, a.f3, a.n, a.sl, a.slen, a.grid,
                                           a.cell3, a.ref_rows, a.ref_nls, a.ref_nlargest,
                                           a.rcutsq, xsi, xsj, a.missing,
                                           ENERGY ? a.epart2 : nullptr, a.run_if);
}

template <typename T>
static void launch_mb_t(const MbArgs& a, bool energy, cudaStream_t st) {
  if (a.n <= 0) return;
  k_mb_short<T><<<nblk(a.n, 4), 128, 0, st>>>(a.pos, a.posf, a.n, a.ld, a.list, a.len, a.grid,
                                              a.rcutsq, a.sl, a.slen, energy ? nullptr : a.run_if);
  const int B = nblk(a.n, 4);
  T* xsi = (T*)a.xsi;
  T* xsj = (T*)a.xsj;
  if (energy) {
    k_mb_pass1<T, true><<<B, 128, 0, st>>>(a.pos, a.posf, a.f3, a.n, a.sl, a.slen, a.grid,
                                           a.ljexist, xsi, xsj, a.epart1, a.eatom, nullptr);
    launch_pass2<T, true>(a, B, xsi, xsj, st);
  } else {
    k_mb_pass1<T, false><<<B, 128, 0, st>>>(a.pos, a.posf, a.f3, a.n, a.sl, a.slen, a.grid,
                                            a.ljexist, xsi, xsj, nullptr, nullptr, a.run_if);
    launch_pass2<T, false>(a, B, xsi, xsj, st);
  }
}

void launch_mb(const MbArgs& a, bool fp32, bool energy, cudaStream_t st) {
  if (fp32)
    launch_mb_t<float>(a, energy, st);
  else
    launch_mb_t<double>(a, energy, st);
}

}  // namespace mdgb
