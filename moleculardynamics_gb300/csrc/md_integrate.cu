// Gear predictor-corrector, accelerations, readyList, thermo reductions and
// the reference's all-pairs potential energy.
//
// predict/correct/accelerations follow cpu/common/Device.cpp:17-133 with the
// reference's roundings (no FMA contraction), so one FP64 step on the GPU
// returns the same bits as the reference on the same forces.  Reductions are
// deterministic: per-block partials in a fixed grid, then one block that sums
// them in a fixed order.
#include <algorithm>
#include <cmath>

#include "mdgb.h"
#include "md_gear.cuh"
#include "md_integrate.h"
#include "md_potential.cuh"

namespace mdgb {

GearCoef gear_coef(double dt) {
  GearCoef k;
  k.c1 = dt;
  k.c2 = k.c1 * dt / 2.0f;
  k.c3 = k.c2 * dt / 3.0f;
  k.c4 = k.c3 * dt / 4.0f;
  k.cr = MD_GEAR1 * k.c2;
  k.cv = MD_GEAR2 * k.c2 / k.c1;
  k.cb = MD_GEAR3 * k.c2 / k.c3;
  k.cc = MD_GEAR4 * k.c2 / k.c4;
  return k;
}

namespace {

__device__ __forceinline__ double mass_of(int type, const Species& sp) {
  return type == SP_N ? (double)sp.mass[0] : (type == SP_O ? (double)sp.mass[1] : (double)sp.mass[2]);
}

__device__ __forceinline__ void skin_check(const GearArgs& a, int i, double x, double y,
                                           double z, int type) {
  if (a.posf) a.posf[i] = make_float4((float)x, (float)y, (float)z, __int_as_float(type));
  if (a.pos_build) {
    float4 pb = a.pos_build[i];
    float dx = (float)x - pb.x, dy = (float)y - pb.y, dz = (float)z - pb.z;
    if (dx * dx + dy * dy + dz * dz > a.trip2) *a.trip = 1;
  }
}

enum { G_PREDICT = 0, G_CORRECT = 1, G_CORRECT_PREDICT = 2 };

// cpu/common/Device.cpp:17-39 (predict) and :44-120 (correct).  EXACT keeps
// every rounding of the reference; otherwise products fuse into FMAs and
// F/m becomes F * (1/m) (the precision form, still FP64 state).
template <int MODE, bool EXACT>
__global__ void __launch_bounds__(256) k_gear(GearArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const GearCoef k = a.k;
  md_double4 r = a.pos[i];
  const int type = (int)r.w;
  double rr[3] = {r.x, r.y, r.z}, v[3], ac[3], b[3], c[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    v[d] = a.vel[3 * i + d];
    ac[d] = a.acc[3 * i + d];
    b[d] = a.b[3 * i + d];
    c[d] = a.c[3 * i + d];
  }
  if (MODE != G_PREDICT) {
    const double mass = mass_of(type, a.sp);
    const double im = type == SP_N ? a.inv_mass[0] : (type == SP_O ? a.inv_mass[1] : a.inv_mass[2]);
    if (EXACT) {
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const double ai = xdiv(a.f3[3 * i + d], mass);
        const double corr = xsub(ai, ac[d]);
        rr[d] = xadd(rr[d], xmul(k.cr, corr));
        v[d] = xadd(v[d], xmul(k.cv, corr));
        ac[d] = ai;
        b[d] = xadd(b[d], xmul(k.cb, corr));
        c[d] = xadd(c[d], xmul(k.cc, corr));
      }
    } else {
      GearAtom s;
      double f[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        s.r[d] = rr[d];
        s.v[d] = v[d];
        s.a[d] = ac[d];
        s.b[d] = b[d];
        s.c[d] = c[d];
        f[d] = a.f3[3 * i + d];
      }
      gear_correct_fma(s, f, im, k);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        rr[d] = s.r[d];
        v[d] = s.v[d];
        ac[d] = s.a[d];
        b[d] = s.b[d];
        c[d] = s.c[d];
      }
    }
    if (MODE == G_CORRECT && a.walls) {
      const double np = a.npos;
      bool hit = false;
      if (rr[0] > np && rr[1] > 0) { hit = true; v[0] = xmul(-v[0], (double)a.energy_loss); rr[0] = np; }
      if (rr[0] > np && rr[1] < 0) { hit = true; rr[0] = -np; }
      if (rr[0] < -np) { hit = true; v[0] = -v[0]; rr[0] = -np; }
      if (fabs(rr[1]) > np) { hit = true; v[1] = -v[1]; rr[1] = xmul(np, xdiv(rr[1], fabs(rr[1]))); }
      if (fabs(rr[2]) > np) { hit = true; v[2] = -v[2]; rr[2] = xmul(np, xdiv(rr[2], fabs(rr[2]))); }
      if (hit) atomicOr(a.wall_flag, 1);
    }
    if (!(isfinite(rr[0]) && isfinite(rr[1]) && isfinite(rr[2]) && isfinite(v[0]) &&
          isfinite(v[1]) && isfinite(v[2])))
      atomicOr(a.status, ST_NONFINITE);
  }
  if (MODE != G_CORRECT) {
    if (EXACT) {
#pragma unroll
      for (int d = 0; d < 3; d++) {
        rr[d] = xadd(xadd(xadd(xadd(rr[d], xmul(k.c1, v[d])), xmul(k.c2, ac[d])),
                          xmul(k.c3, b[d])),
                     xmul(k.c4, c[d]));
        v[d] = xadd(xadd(xadd(v[d], xmul(k.c1, ac[d])), xmul(k.c2, b[d])), xmul(k.c3, c[d]));
        ac[d] = xadd(xadd(ac[d], xmul(k.c1, b[d])), xmul(k.c2, c[d]));
        b[d] = xadd(b[d], xmul(k.c1, c[d]));
      }
    } else {
      GearAtom s;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        s.r[d] = rr[d];
        s.v[d] = v[d];
        s.a[d] = ac[d];
        s.b[d] = b[d];
        s.c[d] = c[d];
      }
      gear_predict_fma(s, k);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        rr[d] = s.r[d];
        v[d] = s.v[d];
        ac[d] = s.a[d];
        b[d] = s.b[d];
      }
    }
  }
#pragma unroll
  for (int d = 0; d < 3; d++) {
    a.vel[3 * i + d] = v[d];
    a.acc[3 * i + d] = ac[d];
    a.b[3 * i + d] = b[d];
    if (MODE != G_PREDICT) a.c[3 * i + d] = c[d];
  }
  r.x = rr[0];
  r.y = rr[1];
  r.z = rr[2];
  a.pos[i] = r;
  skin_check(a, i, rr[0], rr[1], rr[2], type);
}

// cpu/common/Device.cpp:125-133
__global__ void k_accel(const md_double4* __restrict__ pos, double* __restrict__ acc,
                        const double* __restrict__ f3, int n, Species sp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double mass = mass_of((int)pos[i].w, sp);
#pragma unroll
  for (int d = 0; d < 3; d++) acc[3 * i + d] = xdiv(f3[3 * i + d], mass);
}

__global__ void k_posf(const md_double4* __restrict__ pos, float4* __restrict__ posf, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  md_double4 p = pos[i];
  posf[i] = make_float4((float)p.x, (float)p.y, (float)p.z, __int_as_float((int)p.w));
}

__device__ __forceinline__ unsigned long long warp_umax(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long y = __shfl_xor_sync(0xffffffffu, v, o);
    v = y > v ? y : v;
  }
  return v;
}

// cpu/cpumd/Host.cpp:245-271 (max over atoms is exact in any order)
__global__ void k_ready(const md_double4* __restrict__ pos, const double* __restrict__ vel,
                        int n, unsigned long long* umax, int* status) {
  unsigned long long vm = 0, bm = 0;
  bool bad = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    double s = sqrt(norm2_exact(vx, vy, vz));
    md_double4 p = pos[i];
    double b = fmax(fabs(p.x), fmax(fabs(p.y), fabs(p.z)));
    if (!(isfinite(s) && isfinite(b))) {
      bad = true;
      continue;
    }
    unsigned long long us = __double_as_longlong(s), ub = __double_as_longlong(b);
    vm = us > vm ? us : vm;
    bm = ub > bm ? ub : bm;
  }
  vm = warp_umax(vm);
  bm = warp_umax(bm);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&umax[0], vm);
    atomicMax(&umax[1], bm);
  }
  if (bad) atomicOr(status, ST_NONFINITE);
}

constexpr int kRedBlocks = 1024;
constexpr int kRedThreads = 256;

template <int NV>
__device__ __forceinline__ void block_store(double (&v)[NV], double* out) {
  __shared__ double sm[NV][kRedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
    for (int w = 0; w < kRedThreads / 32; w++) s += sm[threadIdx.x][w];
    out[NV * blockIdx.x + threadIdx.x] = s;
  }
}

// block sum of NV doubles into the shared array out[NV] (all threads see it
// after a barrier)
template <int NV>
__device__ __forceinline__ void block_sum_shared(double (&v)[NV], double* out) {
  __shared__ double sm[NV][kRedThreads / 32];
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
    out[threadIdx.x] = s;
  }
}

// common/DebugCalculations.cpp:81-110
__global__ void k_thermo1(const md_double4* __restrict__ pos, const double* __restrict__ vel,
                          int n, Species sp, double* part) {
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    md_double4 p = pos[i];
    const double m = mass_of((int)p.w, sp);
    const double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    v[0] += m * norm2_exact(vx, vy, vz);
    v[1] += m * vx;
    v[2] += m * vy;
    v[3] += m * vz;
    v[4] += m;
    v[5] += m * p.x;
    v[6] += m * p.y;
    v[7] += m * p.z;
  }
  block_store<8>(v, part);
}

// common/DebugCalculations.cpp:124-141 (needs the momentum sums)
__global__ void k_thermo2(const md_double4* __restrict__ pos, const double* __restrict__ vel,
                          int n, Species sp, const double* __restrict__ s8, double* part) {
  const double tot = s8[4];
  const double cx = s8[1] / tot, cy = s8[2] / tot, cz = s8[3] / tot;
  double v[1] = {0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double m = mass_of((int)pos[i].w, sp);
    const double dx = vel[3 * i] - cx, dy = vel[3 * i + 1] - cy, dz = vel[3 * i + 2] - cz;
    v[0] += m * norm2_exact(dx, dy, dz);
  }
  block_store<1>(v, part);
}

__global__ void k_thermo_final(const double* __restrict__ s8, const double* __restrict__ t1,
                               int n, double* out) {
  if (threadIdx.x || blockIdx.x) return;
  const double tot = s8[4];
  out[0] = s8[5] / tot;
  out[1] = s8[6] / tot;
  out[2] = s8[7] / tot;
  out[3] = s8[0] / 2;
  out[4] = s8[1];
  out[5] = s8[2];
  out[6] = s8[3];
  out[7] = t1[0] / (3.0f * ((double)n) * MD_KB);
}

__global__ void k_sum_partials(const double* __restrict__ part, int nblocks, int nv,
                               double* out) {
  __shared__ double sm[kRedThreads];
  for (int k = 0; k < nv; k++) {
    double s = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += part[(size_t)nv * b + k];
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = sm[0];
    __syncthreads();
  }
}

// common/DebugCalculations.cpp:129-270: one block per atom i
__global__ void k_ref_potential(const md_double4* __restrict__ pos, int n, Species sp,
                                double* part) {
  const int i = blockIdx.x;
  const md_double4 pi = pos[i];
  const int ti = (int)pi.w;
  double v[2] = {0, 0};
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    if (j == i) continue;
    const md_double4 pj = pos[j];
    const int tj = (int)pj.w;
    const double ijx = pi.x - pj.x, ijy = pi.y - pj.y, ijz = pi.z - pj.z;
    const double rijsq = norm2_exact(ijx, ijy, ijz);
    if (tj == SP_NG || ti == SP_NG) {
      const int sel = lj_select(ti, tj);
      const double sig = sp.sig[sel], eps = sp.eps[sel];
      double sr2 = sig * sig / rijsq;
      double sr6 = sr2 * sr2 * sr2;
      v[0] += 2.0f * eps * (sr6 * sr6 - sr6);
    } else {
      double va = 0, dva, vr = 0, dvr, vdw, dvdw, bo = 0;
      const double rij = sqrt(rijsq);
      if (rij > MD_CUTOFF_RIJ) continue;
      double fcut, dfcut;
      cutoff<double>(rij / 10, fcut, dfcut);
      if (fcut > 0) {
        const double de = get_de<double>(ti, tj), re = get_re<double>(ti, tj),
                     beta = get_beta<double>(ti, tj);
        attractive<double>(va, dva, rij, de, beta, re);
        repulsive<double>(vr, dvr, rij, de, beta, re);
        const double E = exp(MD_LAMDA3 * (rij - re));
        double xsi = 0, xsj = 0;
        for (int m = 0; m < n; m++) {
          const md_double4 pm = pos[m];
          if ((int)pm.w == SP_NG || m == j || m == i) continue;
          const double imx = pi.x - pm.x, imy = pi.y - pm.y, imz = pi.z - pm.z;
          const double rim = sqrt(norm2_exact(imx, imy, imz));
          const double jmx = pj.x - pm.x, jmy = pj.y - pm.y, jmz = pj.z - pm.z;
          const double rjm = sqrt(norm2_exact(jmx, jmy, jmz));
          double fci, dfci, fcj, dfcj;
          cutoff<double>(rim, fci, dfci);
          cutoff<double>(rjm, fcj, dfcj);
          if (fci > 0) {
            double g, gp;
            angular<double>((rij * rij + rim * rim - rjm * rjm) / (2.0f * rij * rim), g, gp);
            xsi += fci * g * E;
          }
          if (fcj > 0) {
            double g, gp;
            angular<double>((rij * rij + rjm * rjm - rim * rim) / (2.0f * rij * rjm), g, gp);
            xsj += fcj * g * E;
          }
        }
        bo = 0.5f * (1.0f / (1.0f + xsi) + 1.0f / (1.0f + xsj));
      }
      vander_waals<double>(vdw, dvdw, rij, get_r0v<double>(ti, tj));
      v[1] += 0.5f * ((vr - bo * va) + vdw);
    }
  }
  __shared__ double sm[2][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < 2; k++) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sm[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sm[threadIdx.x][w];
    part[2 * i + threadIdx.x] = s;
  }
}

// ---- records in the reference's summation order ----
// PerformCalculations (common/DebugCalculations.cpp:46-124) by one thread,
// atom after atom in the caller's numbering (inv: caller index -> stored
// position, NULL when stored in it), every product and sum rounded on its
// own: the reference's bits.  Output as k_thermo_final.
__global__ void k_thermo_seq(const md_double4* __restrict__ pos, const double* __restrict__ vel,
                             const int* __restrict__ inv, int n, Species sp, double* out) {
  if (threadIdx.x || blockIdx.x) return;
  double mass = 0, cmvx = 0, cmvy = 0, cmvz = 0, total = 0, ke = 0, temp = 0;
  double cx = 0, cy = 0, cz = 0;
  for (int i = 0; i < n; i++) {
    const int p = inv ? inv[i] : i;
    const md_double4 r = pos[p];
    const int t = (int)r.w;
    // :65-76, a switch without a default: another type keeps the last mass
    if (t == SP_N || t == SP_O || t == SP_NG) mass = (double)sp.mass[t];
    const double vx = vel[3 * (size_t)p], vy = vel[3 * (size_t)p + 1],
                 vz = vel[3 * (size_t)p + 2];
    ke = xadd(ke, xmul(mass, xadd(xadd(xmul(vx, vx), xmul(vy, vy)), xmul(vz, vz))));
    cmvx = xadd(cmvx, xmul(mass, vx));
    cmvy = xadd(cmvy, xmul(mass, vy));
    cmvz = xadd(cmvz, xmul(mass, vz));
    total = xadd(total, mass);
    cx = xadd(cx, xmul(mass, r.x));
    cy = xadd(cy, xmul(mass, r.y));
    cz = xadd(cz, xmul(mass, r.z));
  }
  out[0] = xdiv(cx, total);
  out[1] = xdiv(cy, total);
  out[2] = xdiv(cz, total);
  out[4] = cmvx;
  out[5] = cmvy;
  out[6] = cmvz;
  cmvx = xdiv(cmvx, total);
  cmvy = xdiv(cmvy, total);
  cmvz = xdiv(cmvz, total);
  for (int i = 0; i < n; i++) {
    const int p = inv ? inv[i] : i;
    const int t = (int)pos[p].w;
    const double m = (double)sp.mass[t == SP_N ? SP_N : (t == SP_O ? SP_O : SP_NG)];
    const double dx = xsub(vel[3 * (size_t)p], cmvx), dy = xsub(vel[3 * (size_t)p + 1], cmvy),
                 dz = xsub(vel[3 * (size_t)p + 2], cmvz);
    temp = xadd(temp, xmul(m, xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz))));
  }
  out[7] = xdiv(temp, xmul(xmul(3.0, (double)n), (double)MD_KB));
  out[3] = xdiv(ke, 2.0);
}

// The terms of calculatePotentional (common/DebugCalculations.cpp:129-270)
// for the ordered pairs (i, j) of rows [row0, row0 + rows), j fastest, in
// the caller's numbering: the LJ term with every rounding of the reference
// (so an LJ system's sum is bit-identical), the bond-order term as
// k_ref_potential computes it; 0 where the reference adds nothing (i = j,
// a pair of the other kind, beyond CUTOFF_RIJ), which leaves a running sum
// unchanged.
__global__ void k_ref_terms(const md_double4* __restrict__ pos, const int* __restrict__ inv,
                            int n, Species sp, int row0, int rows, double* __restrict__ tlj,
                            double* __restrict__ tmb) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long long)rows * n) return;
  const int i = row0 + (int)(k / n), j = (int)(k % n);
  double elj = 0.0, emb = 0.0;
  if (i != j) {
    const md_double4 pi = pos[inv ? inv[i] : i], pj = pos[inv ? inv[j] : j];
    const int ti = (int)pi.w, tj = (int)pj.w;
    const double ijx = xsub(pi.x, pj.x), ijy = xsub(pi.y, pj.y), ijz = xsub(pi.z, pj.z);
    const double rijsq = norm2_exact(ijx, ijy, ijz);
    if (tj == SP_NG || ti == SP_NG) {
      const int sel = lj_select(ti, tj);
      const double sig = sp.sig[sel], eps = sp.eps[sel];
      const double sr2 = xdiv(xmul(sig, sig), rijsq);
      const double sr6 = xmul(xmul(sr2, sr2), sr2);
      elj = xmul(xmul(2.0, eps), xsub(xmul(sr6, sr6), sr6));
    } else {
      const double rij = sqrt(rijsq);
      if (!(rij > MD_CUTOFF_RIJ)) {
        double va = 0, dva, vr = 0, dvr, vdw, dvdw, bo = 0, fcut, dfcut;
        cutoff<double>(rij / 10, fcut, dfcut);
        if (fcut > 0) {
          const double de = get_de<double>(ti, tj), re = get_re<double>(ti, tj),
                       beta = get_beta<double>(ti, tj);
          attractive<double>(va, dva, rij, de, beta, re);
          repulsive<double>(vr, dvr, rij, de, beta, re);
          const double E = exp(MD_LAMDA3 * (rij - re));
          double xsi = 0, xsj = 0;
          for (int m = 0; m < n; m++) {
            const md_double4 pm = pos[inv ? inv[m] : m];
            if ((int)pm.w == SP_NG || m == j || m == i) continue;
            const double rim = sqrt(norm2_exact(pi.x - pm.x, pi.y - pm.y, pi.z - pm.z));
            const double rjm = sqrt(norm2_exact(pj.x - pm.x, pj.y - pm.y, pj.z - pm.z));
            double fci, dfci, fcj, dfcj;
            cutoff<double>(rim, fci, dfci);
            cutoff<double>(rjm, fcj, dfcj);
            if (fci > 0) {
              double g, gp;
              angular<double>((rij * rij + rim * rim - rjm * rjm) / (2.0f * rij * rim), g, gp);
              xsi += fci * g * E;
            }
            if (fcj > 0) {
              double g, gp;
              angular<double>((rij * rij + rjm * rjm - rim * rim) / (2.0f * rij * rjm), g, gp);
              xsj += fcj * g * E;
            }
          }
          bo = 0.5f * (1.0f / (1.0f + xsi) + 1.0f / (1.0f + xsj));
        }
        vander_waals<double>(vdw, dvdw, rij, get_r0v<double>(ti, tj));
        emb = 0.5f * ((vr - bo * va) + vdw);
      }
    }
  }
  tlj[k] = elj;
  tmb[k] = emb;
}

// The reference's running sums (*vibLJ += ..., *vibMB += ...) over a chunk of
// terms in order, by one thread; out[0..1] carry from chunk to chunk.
__global__ void k_ref_sum_seq(const double* __restrict__ tlj, const double* __restrict__ tmb,
                              long long count, double* out) {
  if (threadIdx.x || blockIdx.x) return;
  double a = out[0], b = out[1];
  for (long long k = 0; k < count; k++) {
    a = xadd(a, tlj[k]);
    b = xadd(b, tmb[k]);
  }
  out[0] = a;
  out[1] = b;
}

__global__ void k_record(const double* __restrict__ th8, const double* __restrict__ elj,
                         const double* __restrict__ emb, const double* __restrict__ ref2,
                         int use_ref, double time, double step, double* rec) {
  if (threadIdx.x || blockIdx.x) return;
  // common/DebugCalculations.cpp:41-50
  const double eu = use_ref ? (ref2[1] + ref2[0]) : (emb[0] + elj[0]);
  rec[0] = time;
  rec[1] = th8[7];
  rec[2] = th8[3] + eu;
  rec[3] = th8[3];
  rec[4] = eu;
  rec[5] = th8[0];
  rec[6] = th8[1];
  rec[7] = th8[2];
  rec[8] = th8[4];
  rec[9] = th8[5];
  rec[10] = th8[6];
  rec[11] = elj[0];
  rec[12] = elj[1];
  rec[13] = emb[0];
  rec[14] = elj[2] + emb[1] + emb[2];
  rec[15] = step;
}

// One record per replica: PerformCalculations (common/DebugCalculations.cpp:
// 46-124) over the replica's atoms [r0, r0 + rn), with its LJ energies e3.
__global__ void __launch_bounds__(kRedThreads)
    k_rep_record(const md_double4* __restrict__ pos, const double* __restrict__ vel,
                 const int* __restrict__ ranges, Species sp, const double* __restrict__ e3,
                 double time, double step, double* __restrict__ rec) {
  const int k = blockIdx.x;
  const int r0 = ranges[2 * k], rn = ranges[2 * k + 1];
  __shared__ double s8[8];
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = r0 + threadIdx.x; i < r0 + rn; i += blockDim.x) {
    const md_double4 p = pos[i];
    const double m = mass_of((int)p.w, sp);
    const double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    v[0] += m * norm2_exact(vx, vy, vz);
    v[1] += m * vx;
    v[2] += m * vy;
    v[3] += m * vz;
    v[4] += m;
    v[5] += m * p.x;
    v[6] += m * p.y;
    v[7] += m * p.z;
  }
  block_sum_shared<8>(v, s8);
  __syncthreads();
  const double tot = s8[4];
  const double cx = s8[1] / tot, cy = s8[2] / tot, cz = s8[3] / tot;
  double w[1] = {0};
  for (int i = r0 + threadIdx.x; i < r0 + rn; i += blockDim.x) {
    const double m = mass_of((int)pos[i].w, sp);
    const double dx = vel[3 * i] - cx, dy = vel[3 * i + 1] - cy, dz = vel[3 * i + 2] - cz;
    w[0] += m * norm2_exact(dx, dy, dz);
  }
  __shared__ double t1[1];
  block_sum_shared<1>(w, t1);
  __syncthreads();
  if (threadIdx.x) return;
  double* o = rec + 16 * (size_t)k;
  const double ek = s8[0] / 2, eu = e3[3 * k];
  o[0] = time;
  o[1] = t1[0] / (3.0f * ((double)rn) * MD_KB);
  o[2] = ek + eu;
  o[3] = ek;
  o[4] = eu;
  o[5] = s8[5] / tot;
  o[6] = s8[6] / tot;
  o[7] = s8[7] / tot;
  o[8] = s8[1];
  o[9] = s8[2];
  o[10] = s8[3];
  o[11] = e3[3 * k];
  o[12] = e3[3 * k + 1];
  o[13] = 0.0;
  o[14] = e3[3 * k + 2];
  o[15] = step;
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }


// ---- equi: Maxwell-Boltzmann velocities (cpu/equi/Host.cpp:416-572) ----

// splitmix64 finaliser (Vigna): one 64-bit hash per (seed, atom, component)
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// uniform on the open interval (0, 1) with 2^32 levels, as (rand() + 1) /
// (RAND_MAX + 2) of cpu/equi/Host.h:26
__device__ __forceinline__ double equi_uniform(unsigned long long seed, int atom, int comp) {
  const unsigned long long z =
      mix64(seed + (3ull * (unsigned long long)atom + (unsigned long long)comp + 1ull) *
                       0x9E3779B97F4A7C15ull);
  return ((double)(unsigned)(z >> 32) + 1.0) / 4294967297.0;
}

// ---- the reference's inverse error function (cpu/equi/Statistics.cpp) ----
// The same steps as the reference, so that velocities drawn here match
// equi's for the same uniforms: Newton iterations on the file's own erf and
// erfc (not CUDA's), every product and sum rounded on its own (no FMA
// contraction), the library's exp, log and sqrt.  The reference's erf stops
// its series after two terms for negative arguments (its stopping test
// divides by the negative sum), so inverf is inaccurate below zero; kept.
// Each loop also stops after kRefIters rounds, which the reference's
// convergence tests reach long before.
constexpr int kRefIters = 400;

// Statistics.cpp:175-196, |x| <= 2.2: the Taylor series
__device__ double ref_erf_series(double x) {
  const double two_sqrtpi = 1.128379167095512574;
  double sum = x, term = x;
  const double xsqr = xmul(x, x);
  int j = 1;
  for (int it = 0; it < kRefIters; it++) {
    term = xmul(term, xdiv(xsqr, (double)j));
    sum = xsub(sum, xdiv(term, (double)(2 * j + 1)));
    ++j;
    term = xmul(term, xdiv(xsqr, (double)j));
    sum = xadd(sum, xdiv(term, (double)(2 * j + 1)));
    ++j;
    if (!(xdiv(fabs(term), sum) > 1e-12)) break;
  }
  return xmul(two_sqrtpi, sum);
}

// Statistics.cpp:209-227, x >= 2.2: the continued fraction
__device__ double ref_erfc_cf(double x) {
  const double one_sqrtpi = 0.564189583547756287;
  double a = 1, b = x, c = x, d = xadd(xmul(x, x), 0.5), q1, q2 = xdiv(b, d), nn = 1.0, t;
  for (int it = 0; it < kRefIters; it++) {
    t = xadd(xmul(a, nn), xmul(b, x));
    a = b;
    b = t;
    t = xadd(xmul(c, nn), xmul(d, x));
    c = d;
    d = t;
    nn = xadd(nn, 0.5);
    q1 = q2;
    q2 = xdiv(b, d);
    if (!(xdiv(fabs(xsub(q1, q2)), q2) > 1e-12)) break;
  }
  return xmul(xmul(one_sqrtpi, exp(xmul(-x, x))), q2);
}

// Statistics.cpp:199-208 erfc
__device__ double ref_erfc(double x) {
  if (fabs(x) < 2.2) return xsub(1.0, ref_erf_series(x));
  if (x < 0) return xsub(2.0, ref_erfc_cf(-x));
  return ref_erfc_cf(x);
}

// Statistics.cpp:175-180 erf
__device__ double ref_erf(double x) {
  if (fabs(x) > 2.2) return xsub(1.0, ref_erfc(x));
  return ref_erf_series(x);
}

// Statistics.cpp:25-41
__device__ double ref_inv_erf_small(double z) {
  const double c = 1.1283791670955125738961589;
  double f = -z, f1 = c;
  double q = xdiv(f, f1), x = -q, x0 = 0;
  for (int it = 0; it < kRefIters && fabs(xsub(x, x0)) > 1e-12 && fabs(f) > 1e-14; it++) {
    x0 = x;
    f = xsub(ref_erf(x), z);
    f1 = xmul(c, exp(xmul(-x, x)));
    q = xdiv(f, f1);
    x = xsub(x, xmul(q, xsub(1.0, xmul(x, q))));
  }
  return x;
}

// Statistics.cpp:58-64 and :74-95
__device__ double ref_inv_erfc_small(double z) {
  const double c = 1.7724538509055160272981675;
  double f = 1;
  const double logz = log(xdiv(1.0, xmul(c, z)));
  const double slz = sqrt(logz);
  const double a = xsub(slz, xdiv(xmul(0.25, log(logz)), slz));
  double x = xdiv(ref_erfc(a), xmul(xmul(xmul(c, a), z), z)), x0 = 0;
  for (int it = 0; it < kRefIters && fabs(xsub(x, x0)) > xmul(1e-12, x) &&
                   fabs(f) > xmul(1e-15, z);
       it++) {
    x0 = x;
    const double slx = sqrt(log(x));
    f = xsub(z, ref_erfc(slx));
    const double f1i = xmul(xmul(xmul(c, x), x), slx);
    x = xsub(x, xmul(xmul(f, f1i),
                     xsub(1.0, xmul(xmul(xmul(c, f), x), xadd(slx, xdiv(0.25, slx))))));
  }
  return sqrt(log(x));
}

// Statistics.cpp:115-140 inverf
__device__ double ref_inverf(double z) {
  const double az = fabs(z);
  if (az >= 1) return z == 1 ? (double)INFINITY : (z == -1 ? -(double)INFINITY : (double)NAN);
  if (az < 0.8125) return ref_inv_erf_small(z);
  if (z > 0) return ref_inv_erfc_small(xsub(1.0, z));
  return -ref_inv_erfc_small(xadd(z, 1.0));
}

// Draws of :438-472 and the momentum sums of :474-478.  Many-body atoms come
// in pairs (i, i + 1), i even and below n_mb, that share one draw made with
// the first atom's mass; the sums count a pair once, with that mass, so
// totalm leaves out the second atoms' masses.  The z draw applies inverf
// before the affine map (:457-461).
__global__ void k_equi_sample(const md_double4* __restrict__ pos, double* __restrict__ vel,
                              const int* __restrict__ orig, int n, int n_mb, Species sp,
                              double temp, unsigned long long seed, double* part) {
  double v[4] = {0, 0, 0, 0};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int i = orig ? orig[p] : p;
    const bool second = i >= 1 && i - 1 < n_mb && ((i - 1) & 1) == 0;
    const bool first = i < n_mb && (i & 1) == 0 && i + 1 < n;
    const int key = second ? i - 1 : i;
    // many-body atoms exist only without the cell order, so p - 1 is i - 1
    const double m = mass_of((int)pos[second ? p - 1 : p].w, sp);
    const double sc = sqrt(xdiv(xmul(2.0, temp), m));
    const double vx = xmul(ref_inverf(xsub(xmul(2.0, equi_uniform(seed, key, 0)), 1.0)), sc);
    const double vy = xmul(ref_inverf(xsub(xmul(2.0, equi_uniform(seed, key, 1)), 1.0)), sc);
    const double vz = xmul(xsub(xmul(2.0, ref_inverf(equi_uniform(seed, key, 2))), 1.0), sc);
    vel[3 * (size_t)p] = vx;
    vel[3 * (size_t)p + 1] = vy;
    vel[3 * (size_t)p + 2] = vz;
    if (!first) {
      v[0] += m * vx;
      v[1] += m * vy;
      v[2] += m * vz;
      v[3] += m;
    }
  }
  block_store<4>(v, part);
}

// :480-484 the shift; :490-512 the sums that follow it (every atom's own mass)
__global__ void k_equi_shift(const md_double4* __restrict__ pos, double* __restrict__ vel, int n,
                             Species sp, double cx, double cy, double cz, double* part) {
  double v[3] = {0, 0, 0};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const double m = mass_of((int)pos[p].w, sp);
    const double vx = vel[3 * (size_t)p] - cx, vy = vel[3 * (size_t)p + 1] - cy,
                 vz = vel[3 * (size_t)p + 2] - cz;
    vel[3 * (size_t)p] = vx;
    vel[3 * (size_t)p + 1] = vy;
    vel[3 * (size_t)p + 2] = vz;
    v[0] += vx * m;
    v[1] += vy * m;
    v[2] += vz * m;
  }
  block_store<3>(v, part);
}

// :519-538 sum m v^2 (the products in the reference's order)
__global__ void k_equi_ke(const md_double4* __restrict__ pos, const double* __restrict__ vel,
                          int n, Species sp, double* part) {
  double v[1] = {0};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const double m = mass_of((int)pos[p].w, sp);
    v[0] += m * norm2_exact(vel[3 * (size_t)p], vel[3 * (size_t)p + 1], vel[3 * (size_t)p + 2]);
  }
  block_store<1>(v, part);
}

__global__ void k_equi_scale(double* __restrict__ vel, int n3, double s) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n3; k += gridDim.x * blockDim.x)
    vel[k] *= s;
}

}  // namespace

void launch_predict(const GearArgs& a, cudaStream_t st) {
  if (a.n <= 0) return;
  if (a.exact)
    k_gear<G_PREDICT, true><<<nblk(a.n, 256), 256, 0, st>>>(a);
  else
    k_gear<G_PREDICT, false><<<nblk(a.n, 256), 256, 0, st>>>(a);
}
void launch_correct(const GearArgs& a, cudaStream_t st) {
  if (a.n <= 0) return;
  if (a.exact)
    k_gear<G_CORRECT, true><<<nblk(a.n, 256), 256, 0, st>>>(a);
  else
    k_gear<G_CORRECT, false><<<nblk(a.n, 256), 256, 0, st>>>(a);
}
void launch_correct_predict(const GearArgs& a, cudaStream_t st) {
  if (a.n <= 0) return;
  if (a.exact)
    k_gear<G_CORRECT_PREDICT, true><<<nblk(a.n, 256), 256, 0, st>>>(a);
  else
    k_gear<G_CORRECT_PREDICT, false><<<nblk(a.n, 256), 256, 0, st>>>(a);
}
void launch_accel(const md_double4* pos, double* acc, const double* f3, int n, Species sp,
                  cudaStream_t st) {
  if (n > 0) k_accel<<<nblk(n, 256), 256, 0, st>>>(pos, acc, f3, n, sp);
}
void launch_posf(const md_double4* pos, float4* posf, int n, cudaStream_t st) {
  if (n > 0) k_posf<<<nblk(n, 256), 256, 0, st>>>(pos, posf, n);
}
void launch_ready(const md_double4* pos, const double* vel, int n, unsigned long long* umax,
                  int* status, cudaStream_t st) {
  cudaMemsetAsync(umax, 0, 2 * sizeof(unsigned long long), st);
  int B = nblk(n, 256);
  if (B > kRedBlocks) B = kRedBlocks;
  if (B > 0) k_ready<<<B, 256, 0, st>>>(pos, vel, n, umax, status);
}
void launch_thermo(const md_double4* pos, const double* vel, int n, Species sp, double* part,
                   double* out, cudaStream_t st) {
  int B = nblk(n, kRedThreads);
  if (B > kRedBlocks) B = kRedBlocks;
  if (B < 1) B = 1;
  double* s8 = part + 8 * kRedBlocks;
  double* t1 = s8 + 8;
  k_thermo1<<<B, kRedThreads, 0, st>>>(pos, vel, n, sp, part);
  k_sum_partials<<<1, kRedThreads, 0, st>>>(part, B, 8, s8);
  k_thermo2<<<B, kRedThreads, 0, st>>>(pos, vel, n, sp, s8, part);
  k_sum_partials<<<1, kRedThreads, 0, st>>>(part, B, 1, t1);
  k_thermo_final<<<1, 32, 0, st>>>(s8, t1, n, out);
}

int equi_velocities(const md_double4* pos, double* vel, const int* orig, int n, int n_mb,
                    Species sp, double temp, unsigned long long seed, double* part,
                    int* iterations, cudaStream_t st) {
  int B = nblk(n, kRedThreads);
  if (B > kRedBlocks) B = kRedBlocks;
  if (B < 1) B = 1;
  double* sums = part + 4 * kRedBlocks;
  double h[4];
  auto reduce = [&](int nv) -> cudaError_t {
    k_sum_partials<<<1, kRedThreads, 0, st>>>(part, B, nv, sums);
    cudaError_t e = cudaMemcpyAsync(h, sums, sizeof(double) * nv, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
  };
  k_equi_sample<<<B, kRedThreads, 0, st>>>(pos, vel, orig, n, n_mb, sp, temp, seed, part);
  cudaError_t e = reduce(4);
  if (e != cudaSuccess) return (int)e;
  const double totalm = h[3];
  double cx = h[0] / totalm, cy = h[1] / totalm, cz = h[2] / totalm;
  // :480-515 until every component is within 1e-15.  The pairs' missing
  // masses leave a residue after the first shift; from then on each shift
  // scales the remainder by minus the ratio of the second atoms' mass to
  // totalm: the loop converges while that ratio is below 1 and never
  // otherwise (the reference then loops forever).  A shift after the second
  // that does not shrink the largest component ends the loop with an error.
  int it = 0;
  double prev = 1e300;
  while (fabs(cx) > 1.0e-15 || fabs(cy) > 1.0e-15 || fabs(cz) > 1.0e-15) {
    const double big = fmax(fabs(cx), fmax(fabs(cy), fabs(cz)));
    if (++it > 100000 || (it > 2 && !(big < prev))) {
      *iterations = it;
      return -1;
    }
    prev = big;
    k_equi_shift<<<B, kRedThreads, 0, st>>>(pos, vel, n, sp, cx, cy, cz, part);
    if ((e = reduce(3)) != cudaSuccess) return (int)e;
    cx = h[0] / totalm;
    cy = h[1] / totalm;
    cz = h[2] / totalm;
  }
  *iterations = it;
  // :519-546 rescale to temp
  k_equi_ke<<<B, kRedThreads, 0, st>>>(pos, vel, n, sp, part);
  if ((e = reduce(1)) != cudaSuccess) return (int)e;
  const double t = h[0] / (3.0 * (double)n);
  const double scalev = sqrt(temp / t);
  k_equi_scale<<<nblk(3 * n, 256), 256, 0, st>>>(vel, 3 * n, scalev);
  return (int)cudaGetLastError();
}

void launch_rep_records(const md_double4* pos, const double* vel, const int* ranges, int nrep,
                        Species sp, const double* e3, double time, double step, double* rec,
                        cudaStream_t st) {
  if (nrep > 0)
    k_rep_record<<<nrep, kRedThreads, 0, st>>>(pos, vel, ranges, sp, e3, time, step, rec);
}
void launch_sum_partials(const double* part, int nblocks, int nv, double* out,
                         cudaStream_t st) {
  k_sum_partials<<<1, kRedThreads, 0, st>>>(part, nblocks, nv, out);
}
void launch_ref_potential(const md_double4* pos, int n, Species sp, double* part, double* out,
                          cudaStream_t st) {
  if (n <= 0) {
    cudaMemsetAsync(out, 0, 2 * sizeof(double), st);
    return;
  }
  k_ref_potential<<<n, 128, 0, st>>>(pos, n, sp, part);
  k_sum_partials<<<1, kRedThreads, 0, st>>>(part, n, 2, out);
}
void launch_thermo_seq(const md_double4* pos, const double* vel, const int* inv, int n,
                       Species sp, double* out, cudaStream_t st) {
  k_thermo_seq<<<1, 32, 0, st>>>(pos, vel, inv, n, sp, out);
}
int launch_ref_potential_seq(const md_double4* pos, const int* inv, int n, Species sp,
                             double* buf, long long buf_terms, double* out, cudaStream_t st) {
  cudaMemsetAsync(out, 0, 2 * sizeof(double), st);
  if (n <= 0) return 0;
  const int rows = (int)std::max(1LL, std::min((long long)n, buf_terms / n));
  int launches = 1;
  for (int r0 = 0; r0 < n; r0 += rows) {
    const int nr = std::min(rows, n - r0);
    const long long terms = (long long)nr * n;
    k_ref_terms<<<nblk(terms, 256), 256, 0, st>>>(pos, inv, n, sp, r0, nr, buf, buf + buf_terms);
    k_ref_sum_seq<<<1, 32, 0, st>>>(buf, buf + buf_terms, terms, out);
    launches += 2;
  }
  return launches;
}
void launch_record(const double* th8, const double* e_lj3, const double* e_mb3,
                   const double* ref2, int use_ref, double time, double step, double* rec16,
                   cudaStream_t st) {
  k_record<<<1, 32, 0, st>>>(th8, e_lj3, e_mb3, ref2, use_ref, time, step, rec16);
}

}  // namespace mdgb

namespace {

__global__ void k_conv_selftest(const float* f, const double* d, int n, double* w, double* wr,
                                float* nr, float* nrr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  w[i] = mdgb::widen_exact(f[i]);
  wr[i] = (double)f[i];
  nr[i] = mdgb::narrow_rn(d[i]);
  nrr[i] = __double2float_rn(d[i]);
}

}  // namespace

extern "C" md_status mdgb_conv_selftest(const float* f, const double* d, int count, double* wide,
                                        double* wide_ref, float* narrow, float* narrow_ref) {
  if (count <= 0 || !f || !d || !wide || !wide_ref || !narrow || !narrow_ref)
    return MD_BAD_ARGUMENT;
  const size_t n = (size_t)count;
  float* df = nullptr;
  double* dd = nullptr;
  if (cudaMalloc(&df, n * sizeof(float) * 3) != cudaSuccess) return MD_CUDA_ERROR;
  if (cudaMalloc(&dd, n * sizeof(double) * 3) != cudaSuccess) {
    cudaFree(df);
    return MD_CUDA_ERROR;
  }
  float* dn = df + n;
  float* dnr = dn + n;
  double* dw = dd + n;
  double* dwr = dw + n;
  md_status r = MD_OK;
  if (cudaMemcpy(df, f, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dd, d, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    r = MD_CUDA_ERROR;
  if (r == MD_OK) {
    k_conv_selftest<<<(count + 255) / 256, 256>>>(df, dd, count, dw, dwr, dn, dnr);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(wide, dw, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(wide_ref, dwr, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(narrow, dn, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(narrow_ref, dnr, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
      r = MD_CUDA_ERROR;
  }
  cudaFree(df);
  cudaFree(dd);
  return r;
}
