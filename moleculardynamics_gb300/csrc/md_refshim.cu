// Reference-signature entry points (mdgb_* in include/mdgb.h).
//
// Each function has the arguments and meaning of the reference function it
// replaces (cpu/common/Device.h:19-23, common/NeighborList.h:30,
// common/DebugCalculations.h:18-20) and runs it on the GPU: host arrays are
// copied in, the kernel runs, results are copied back.  Device buffers are
// cached per host thread and grow as needed.  Failures are reported through
// mdgb_last_status() instead of the reference's exit(EXIT_FAILURE).
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/mdgb.h"
#include "md_forces.h"
#include "md_integrate.h"
#include "md_neighbor.cuh"
#include "md_potential.cuh"

using namespace mdgb;

namespace {

struct Shim {
  bool init = false;
  cudaStream_t st = nullptr;
  int species = MD_SPECIES_NEON;
  md_double4* pos = nullptr;
  double* v[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  long long n_alloc = 0;
  int* rows = nullptr;
  long long rows_alloc = 0;
  uint32_t* ell = nullptr;
  int* len = nullptr;
  uint32_t* sl = nullptr;
  int* slen = nullptr;
  double *xsi = nullptr, *xsj = nullptr;
  long long ell_alloc = 0, len_alloc = 0;
  int* flags = nullptr;  // status, wall flag, missing
  Scratch sc;
  double* part = nullptr;
  long long part_alloc = 0;
  double* out = nullptr;
  NeighborList nl;
};

thread_local Shim g_shim;
thread_local int g_last = MD_OK;

Species shim_species(int which) {
  Species s;
  s.sig[0] = 3.015f;
  s.sig[1] = 2.835f;
  s.eps[0] = 0.328e-4f;
  s.eps[1] = 0.447e-4f;
  s.mass[0] = 14.00674f;
  s.mass[1] = 15.9994f;
  if (which == MD_SPECIES_ARGON) {
    s.sig[2] = 3.405f;
    s.eps[2] = 9.960172e-5f;
    s.mass[2] = 39.948f;
  } else {
    s.sig[2] = 2.72f;
    s.eps[2] = 0.391e-4f;
    s.mass[2] = 20.1797f;
  }
  return s;
}

template <typename T>
bool grow(T*& p, long long& have, long long need) {
  if (need <= have && p) return true;
  if (p) cudaFree(p);
  p = nullptr;
  if (need < 1) need = 1;
  if (cudaMalloc(&p, sizeof(T) * (size_t)need) != cudaSuccess) {
    have = 0;
    return false;
  }
  have = need;
  return true;
}

bool shim_ready(long long n) {
  Shim& s = g_shim;
  if (!s.init) {
    if (cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking) != cudaSuccess) return false;
    if (cudaMalloc(&s.flags, sizeof(int) * 4) != cudaSuccess) return false;
    if (cudaMalloc(&s.sc.dpart, sizeof(double) * (8 * 1024 + 64)) != cudaSuccess) return false;
    if (cudaMalloc(&s.sc.umax, sizeof(unsigned long long) * 4) != cudaSuccess) return false;
    if (cudaMalloc(&s.sc.counts, sizeof(int) * 8) != cudaSuccess) return false;
    if (cudaMalloc(&s.out, sizeof(double) * 16) != cudaSuccess) return false;
    s.init = true;
  }
  if (n > s.n_alloc) {
    if (s.pos) cudaFree(s.pos);
    s.pos = nullptr;
    if (cudaMalloc(&s.pos, sizeof(md_double4) * (size_t)n) != cudaSuccess) return false;
    for (double*& p : s.v) {
      if (p) cudaFree(p);
      p = nullptr;
      if (cudaMalloc(&p, sizeof(double) * 3 * (size_t)n) != cudaSuccess) return false;
    }
    s.n_alloc = n;
  }
  return true;
}

bool up(void* d, const void* h, size_t bytes) {
  return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, g_shim.st) == cudaSuccess;
}
bool down(void* h, const void* d, size_t bytes) {
  return cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, g_shim.st) == cudaSuccess;
}
bool finish() {
  if (cudaStreamSynchronize(g_shim.st) != cudaSuccess) return false;
  return cudaGetLastError() == cudaSuccess;
}

#define SHIM_CK(cond, code)        \
  do {                             \
    if (!(cond)) {                 \
      g_last = (code);             \
      return;                      \
    }                              \
  } while (0)

// cpu/common/LennardJones.h:35-93 over rows in the reference layout
__global__ void k_lj_rows(const md_double4* __restrict__ pos, double* __restrict__ f3, int n,
                          int nlargest, int nls, const int* __restrict__ list, double rcutsq,
                          Species sp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const md_double4 pi = pos[i];
  const int ti = (int)pi.w;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  const int* row = list + (size_t)i * nls;
  for (int j = 0; j < nlargest && row[j] != -1; j++) {
    const md_double4 pj = pos[row[j]];
    const double ijx = xsub(pi.x, pj.x), ijy = xsub(pi.y, pj.y), ijz = xsub(pi.z, pj.z);
    const double r2 = norm2_exact(ijx, ijy, ijz);
    if (r2 >= rcutsq) continue;
    const int tj = (int)pj.w;
    if (tj == SP_NG || ti == SP_NG) {
      const int sel = lj_select(ti, tj);
      lj_pair_exact(fx, fy, fz, __dsqrt_rn(r2), ijx, ijy, ijz, sp.sig[sel], sp.eps[sel]);
    }
  }
  f3[3 * i] = fx;
  f3[3 * i + 1] = fy;
  f3[3 * i + 2] = fz;
}

// reference rows -> ELL slot-major rows (candidate order kept)
__global__ void k_rows_to_ell(const int* __restrict__ list, int n, int nlargest, int nls,
                              uint32_t* __restrict__ ell, int* __restrict__ len) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int* row = list + (size_t)i * nls;
  int k = 0;
  for (; k < nlargest && row[k] != -1; k++) ell[(size_t)k * n + i] = (uint32_t)row[k];
  len[i] = k;
}

}  // namespace

extern "C" {

int mdgb_last_status(void) { return g_last; }

void mdgb_set_species(int species) {
  g_shim.species = species == MD_SPECIES_ARGON ? MD_SPECIES_ARGON : MD_SPECIES_NEON;
}

void mdgb_free(void* p) { free(p); }

void mdgb_predict(double* r4, double* v3, double* a3, double* b3, double* c3, double dt,
                  int nop) {
  g_last = MD_OK;
  SHIM_CK(nop >= 0 && (nop == 0 || (r4 && v3 && a3 && b3 && c3)), MD_BAD_ARGUMENT);
  if (nop == 0) return;
  SHIM_CK(shim_ready(nop), MD_CUDA_ERROR);
  Shim& s = g_shim;
  const size_t N = (size_t)nop;
  SHIM_CK(up(s.pos, r4, 32 * N) && up(s.v[0], v3, 24 * N) && up(s.v[1], a3, 24 * N) &&
              up(s.v[2], b3, 24 * N) && up(s.v[3], c3, 24 * N),
          MD_CUDA_ERROR);
  GearArgs g{};
  g.pos = s.pos;
  g.vel = s.v[0];
  g.acc = s.v[1];
  g.b = s.v[2];
  g.c = s.v[3];
  g.n = nop;
  g.k = gear_coef(dt);
  g.sp = shim_species(s.species);
  g.status = s.flags;
  g.exact = 1;
  launch_predict(g, s.st);
  SHIM_CK(down(r4, s.pos, 32 * N) && down(v3, s.v[0], 24 * N) && down(a3, s.v[1], 24 * N) &&
              down(b3, s.v[2], 24 * N) && finish(),
          MD_CUDA_ERROR);
}

void mdgb_correct(double* r4, double* v3, const double* f3, double* a3, double* b3,
                  double* c3, double dt, int nop, double npos, int* flag, float energy_loss) {
  g_last = MD_OK;
  SHIM_CK(nop >= 0 && flag && (nop == 0 || (r4 && v3 && f3 && a3 && b3 && c3)), MD_BAD_ARGUMENT);
  *flag = 0;
  if (nop == 0) return;
  SHIM_CK(shim_ready(nop), MD_CUDA_ERROR);
  Shim& s = g_shim;
  const size_t N = (size_t)nop;
  SHIM_CK(up(s.pos, r4, 32 * N) && up(s.v[0], v3, 24 * N) && up(s.v[1], a3, 24 * N) &&
              up(s.v[2], b3, 24 * N) && up(s.v[3], c3, 24 * N) && up(s.v[4], f3, 24 * N),
          MD_CUDA_ERROR);
  SHIM_CK(cudaMemsetAsync(s.flags, 0, sizeof(int) * 4, s.st) == cudaSuccess, MD_CUDA_ERROR);
  GearArgs g{};
  g.pos = s.pos;
  g.vel = s.v[0];
  g.acc = s.v[1];
  g.b = s.v[2];
  g.c = s.v[3];
  g.f3 = s.v[4];
  g.n = nop;
  g.k = gear_coef(dt);
  g.sp = shim_species(s.species);
  g.status = s.flags;
  g.npos = npos;
  g.energy_loss = energy_loss;
  g.walls = 1;
  g.wall_flag = s.flags + 1;
  g.exact = 1;
  launch_correct(g, s.st);
  int fl[2] = {0, 0};
  SHIM_CK(down(r4, s.pos, 32 * N) && down(v3, s.v[0], 24 * N) && down(a3, s.v[1], 24 * N) &&
              down(b3, s.v[2], 24 * N) && down(c3, s.v[3], 24 * N) &&
              down(fl, s.flags, sizeof(fl)) && finish(),
          MD_CUDA_ERROR);
  *flag = fl[1] ? 1 : 0;
}

void mdgb_lennard_jones_forces(const double* pos4, double* f3, int n, int nlargestsize,
                               int nlistsize, const int* list, double rcutsq) {
  g_last = MD_OK;
  SHIM_CK(n >= 0 && (n == 0 || (pos4 && f3)) && nlistsize >= 0, MD_BAD_ARGUMENT);
  if (n == 0) return;
  SHIM_CK(nlistsize == 0 || list, MD_BAD_ARGUMENT);
  SHIM_CK(shim_ready(n), MD_CUDA_ERROR);
  Shim& s = g_shim;
  const long long nrows = (long long)n * nlistsize;
  SHIM_CK(grow(s.rows, s.rows_alloc, nrows), MD_OUT_OF_MEMORY);
  SHIM_CK(up(s.pos, pos4, 32 * (size_t)n), MD_CUDA_ERROR);
  if (nrows) SHIM_CK(up(s.rows, list, sizeof(int) * (size_t)nrows), MD_CUDA_ERROR);
  k_lj_rows<<<(n + 127) / 128, 128, 0, s.st>>>(s.pos, s.v[4], n, nlistsize ? nlargestsize : 0,
                                               nlistsize, s.rows, rcutsq,
                                               shim_species(s.species));
  SHIM_CK(down(f3, s.v[4], 24 * (size_t)n) && finish(), MD_CUDA_ERROR);
}

void mdgb_many_body_forces(const double* pos4, double* f3, int n, int nlargestsize,
                           int nlistsize, const int* list, double rcutsq, int ljexist) {
  g_last = MD_OK;
  SHIM_CK(n >= 0 && (n == 0 || (pos4 && f3)) && nlistsize >= 0, MD_BAD_ARGUMENT);
  if (n == 0) return;
  SHIM_CK(nlistsize == 0 || list, MD_BAD_ARGUMENT);
  SHIM_CK(shim_ready(n), MD_CUDA_ERROR);
  Shim& s = g_shim;
  const long long nrows = (long long)n * nlistsize;
  const int cap = nlargestsize > 0 ? nlargestsize : 1;
  const long long ell = (long long)cap * n;
  SHIM_CK(grow(s.rows, s.rows_alloc, nrows) && grow(s.ell, s.ell_alloc, ell), MD_OUT_OF_MEMORY);
  // short list and xi scratch sized like the ELL rows
  static thread_local long long sl_alloc = 0, x_alloc = 0, xj_alloc = 0;
  SHIM_CK(grow(s.sl, sl_alloc, ell) && grow(s.xsi, x_alloc, ell) && grow(s.xsj, xj_alloc, ell) &&
              grow(s.len, s.len_alloc, n),
          MD_OUT_OF_MEMORY);
  static thread_local long long slen_alloc = 0;
  SHIM_CK(grow(s.slen, slen_alloc, n), MD_OUT_OF_MEMORY);
  SHIM_CK(up(s.pos, pos4, 32 * (size_t)n), MD_CUDA_ERROR);
  if (nrows) SHIM_CK(up(s.rows, list, sizeof(int) * (size_t)nrows), MD_CUDA_ERROR);
  if (ljexist) SHIM_CK(up(s.v[4], f3, 24 * (size_t)n), MD_CUDA_ERROR);
  SHIM_CK(cudaMemsetAsync(s.flags, 0, sizeof(int) * 4, s.st) == cudaSuccess, MD_CUDA_ERROR);
  k_rows_to_ell<<<(n + 127) / 128, 128, 0, s.st>>>(s.rows, n, nlistsize ? nlargestsize : 0,
                                                   nlistsize, s.ell, s.len);
  MbArgs a{};
  a.pos = s.pos;
  a.posf = nullptr;
  a.f3 = s.v[4];
  a.n = n;
  a.list = s.ell;
  a.len = s.len;
  a.ld = n;
  a.grid = Grid{};
  a.cell3 = nullptr;
  a.ref_rows = s.rows;
  a.ref_nls = nlistsize;
  a.ref_nlargest = nlistsize ? nlargestsize : 0;
  a.rcutsq = rcutsq;
  a.ljexist = ljexist;
  a.sl = s.sl;
  a.slen = s.slen;
  a.xsi = s.xsi;
  a.xsj = s.xsj;
  a.missing = s.flags + 2;
  launch_mb(a, false, false, s.st);
  SHIM_CK(down(f3, s.v[4], 24 * (size_t)n) && finish(), MD_CUDA_ERROR);
}

void mdgb_calculate_accelerations(const double* pos4, double* a3, const double* f3, int n) {
  g_last = MD_OK;
  SHIM_CK(n >= 0 && (n == 0 || (pos4 && a3 && f3)), MD_BAD_ARGUMENT);
  if (n == 0) return;
  SHIM_CK(shim_ready(n), MD_CUDA_ERROR);
  Shim& s = g_shim;
  SHIM_CK(up(s.pos, pos4, 32 * (size_t)n) && up(s.v[4], f3, 24 * (size_t)n), MD_CUDA_ERROR);
  launch_accel(s.pos, s.v[1], s.v[4], n, shim_species(s.species), s.st);
  SHIM_CK(down(a3, s.v[1], 24 * (size_t)n) && finish(), MD_CUDA_ERROR);
}

int* mdgb_build_neighbor_list(const double* pos4, mdgb_list_settings* ls, double box,
                              int buckets, int n) {
  g_last = MD_OK;
  (void)buckets;  // the GPU cell table sizes itself; rows do not depend on it
  if (!ls || n < 0 || (n > 0 && !pos4)) {
    g_last = MD_BAD_ARGUMENT;
    return nullptr;
  }
  if (!shim_ready(n > 0 ? n : 1)) {
    g_last = MD_CUDA_ERROR;
    return nullptr;
  }
  Shim& s = g_shim;
  if (n > 0 && !up(s.pos, pos4, 32 * (size_t)n)) {
    g_last = MD_CUDA_ERROR;
    return nullptr;
  }
  cudaMemsetAsync(s.flags, 0, sizeof(int) * 4, s.st);
  std::string err;
  Grid g = make_grid_reference(box, ls->rs);
  int r = list_build(s.nl, s.pos, n, g, 0, 0.f, (double)ls->rcut, s.sc, s.flags, s.st, err);
  if (r != 0) {
    if (r == -1)
      g_last = err.find("non-finite") != std::string::npos ? MD_NONFINITE : MD_CELL_OVERFLOW;
    else
      g_last = MD_CUDA_ERROR;
    return nullptr;
  }
  ls->nlistsize = s.nl.nlistsize;
  ls->nlargestsize = s.nl.nlargest;
  const long long total = (long long)s.nl.nlistsize * n;
  int* out = (int*)malloc(sizeof(int) * (size_t)(total > 0 ? total : 1));
  if (!out) {
    g_last = MD_OUT_OF_MEMORY;
    return nullptr;
  }
  if (total > 0) {
    if (!grow(s.rows, s.rows_alloc, total)) {
      free(out);
      g_last = MD_OUT_OF_MEMORY;
      return nullptr;
    }
    list_reference_rows(s.nl, s.pos, s.rows, nullptr, s.st);
    if (!down(out, s.rows, sizeof(int) * (size_t)total) || !finish()) {
      free(out);
      g_last = MD_CUDA_ERROR;
      return nullptr;
    }
  }
  return out;
}

void mdgb_perform_calculations(const double* pos4, const double* vel3, int n, double* com_x,
                               double* com_y, double* com_z, double* kinetic, double* mom_x,
                               double* mom_y, double* mom_z, double* temp) {
  g_last = MD_OK;
  SHIM_CK(n > 0 && pos4 && vel3, MD_BAD_ARGUMENT);
  SHIM_CK(shim_ready(n), MD_CUDA_ERROR);
  Shim& s = g_shim;
  SHIM_CK(up(s.pos, pos4, 32 * (size_t)n) && up(s.v[0], vel3, 24 * (size_t)n), MD_CUDA_ERROR);
  launch_thermo(s.pos, s.v[0], n, shim_species(s.species), s.sc.dpart, s.out, s.st);
  double o[8];
  SHIM_CK(down(o, s.out, sizeof(o)) && finish(), MD_CUDA_ERROR);
  double* dst[8] = {com_x, com_y, com_z, kinetic, mom_x, mom_y, mom_z, temp};
  for (int k = 0; k < 8; k++)
    if (dst[k]) *dst[k] = o[k];
}

void mdgb_calculate_potential(const double* pos4, double* vib_lj, double* vib_mb, int n) {
  g_last = MD_OK;
  SHIM_CK(n >= 0 && (n == 0 || pos4), MD_BAD_ARGUMENT);
  SHIM_CK(shim_ready(n > 0 ? n : 1), MD_CUDA_ERROR);
  Shim& s = g_shim;
  SHIM_CK(grow(s.part, s.part_alloc, 2LL * (n > 0 ? n : 1)), MD_OUT_OF_MEMORY);
  if (n > 0) SHIM_CK(up(s.pos, pos4, 32 * (size_t)n), MD_CUDA_ERROR);
  launch_ref_potential(s.pos, n, shim_species(s.species), s.part, s.out, s.st);
  double o[2];
  SHIM_CK(down(o, s.out, sizeof(o)) && finish(), MD_CUDA_ERROR);
  if (vib_lj) *vib_lj = o[0];
  if (vib_mb) *vib_mb = o[1];
}

}  // extern "C"
