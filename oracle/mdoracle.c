/*
 * mdoracle.c: CPU restatement of the FP64 MD step of vakuras/moleculardynamics.
 *
 * TEST INFRASTRUCTURE, NOT THE PRODUCT.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline arm load this file's library, as the checker
 * or as the timed CPU baseline.  The GPU engine never calls it.
 *
 * Each function follows the reference function cited above it, with the same
 * expression shapes and the same float-literal promotions, so that, built
 * with -ffp-contract=off, it returns the same bits as the reference compiled
 * in place (pinned by tests/test_oracle_pinned.py).  Differences in structure
 * that do not change results:
 *   - cells are grouped with an open-addressing table of this file's own;
 *     only cell membership and order matter to the rows, not bucket ids;
 *   - the bond-order xi scratch is kept per (i, list slot), not N x N;
 *   - per-atom loops are split over OpenMP threads; every sum stays inside
 *     one atom, so results do not depend on the thread count.
 */
#include "mdoracle.h"

#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants of common/Constants.h:13-79 (float literals, as there) ---- */
#define SP_N 0
#define SP_O 1
#define SP_NG 2
#define reN 1.097f
#define reO 1.2075f
#define reNO 1.15f
#define reNvdw 3.72f
#define reOvdw 3.31f
#define reNOvdw 3.51f
#define sigNvdw 3.31f
#define deN 941.4e-4f
#define deO 493.55309e-4f
#define deNO 626.734e-4f
#define betaN 2.71009f
#define betaO 2.2478f
#define betaNO 2.24068f
#define CUTOFF_RIJ (15 * sigNvdw)
#define CUTOFF_RIJSQ (225 * sigNvdw * sigNvdw)
#define GEAR1 0.15833333333333333333333333333333f
#define GEAR2 0.75f
#define GEAR3 0.5f
#define GEAR4 0.08333333333333333333333333333333f
#define BO_S 2.0f
#define BO_GM 0.3f
#define BO_GMSQ 0.09f
#define BO_ALFAV 3.0f
#define BO_ALFAVSQ 9.0f
#define BO_ALFA 2.0f
#define BO_R0 1.3f
#define BO_LAMDA3 1.33f
#define BO_C 25.f
#define BO_D 4.0417f
#define BO_H 0.0f
#define KB_FLOAT 8.314e-7f

void orc_species_get(int which, orc_species* o) {
  /* common/Constants.h:36-43,55-57 (neon); argon in the NG slot otherwise */
  o->sigNGN = 3.015f;
  o->sigNGO = 2.835f;
  o->epsNGN = 0.328e-4f;
  o->epsNGO = 0.447e-4f;
  o->mN = 14.00674f;
  o->mO = 15.9994f;
  if (which == ORC_SPECIES_ARGON) {
    o->sigNG = 3.405f;
    o->epsNG = 9.960172e-5f;
    o->mNG = 39.948f;
  } else {
    o->sigNG = 2.72f;
    o->epsNG = 0.391e-4f;
    o->mNG = 20.1797f;
  }
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---- getters: common/Getters.cpp:13-78 ---- */
static double get_mass(int id, const orc_species* sp) {
  if (id == SP_N) return sp->mN;
  if (id == SP_O) return sp->mO;
  return sp->mNG;
}
static double get_re(int ti, int tj) {
  if (ti == tj) return ti == SP_N ? reN : reO;
  return reNO;
}
static double get_de(int ti, int tj) {
  if (ti == tj) return ti == SP_N ? deN : deO;
  return deNO;
}
static double get_beta(int ti, int tj) {
  if (ti == tj) return ti == SP_N ? betaN : betaO;
  return betaNO;
}
static double get_r0v(int ti, int tj) {
  if (ti == tj) return ti == SP_N ? reNvdw : reOvdw;
  return reNOvdw;
}

/* ---- common/arvdwfc.cpp:17-59 (T = double) ---- */
static void attractive(double* va, double* dva, double rij, double De, double beta,
                       double re) {
  /* sqrt(2.0f/S) is std::sqrt(float) in the reference: exactly 1.0f */
  const float s2 = sqrtf(2.0f / BO_S);
  *va = BO_S * De / (BO_S - 1.0f) * exp(-beta * s2 * (rij - re));
  *dva = beta * s2 * *va;
}
static void repulsive(double* vr, double* dvr, double rij, double De, double beta,
                      double re) {
  const float s2 = sqrtf(BO_S * 2.0f);
  *vr = De / (BO_S - 1.0f) * exp(-beta * s2 * (rij - re)) +
        7.0e-8f * exp(-10.0f * beta * (rij - re));
  *dvr = beta * sqrtf(2.0f * BO_S) * *vr;
}
static void vander_waals(double* vdw, double* dvdw, double rij, double r0v) {
  double alfavm = BO_ALFAV * (rij - r0v);
  double gmexp = BO_GM * exp(-alfavm);
  double a = exp(alfavm) + gmexp;
  double b = BO_ALFAV * (exp(alfavm) - gmexp);
  double db = BO_ALFAVSQ * a;
  double v = 1.0f + 50.0f * BO_GM + BO_GMSQ + 10.0f * (BO_GM - 1.0f) * b;
  *dvdw = -1.0e-4f * ((10.0f * (BO_GM - 1.0f) * db * a - 2.0f * b * v) / (a * a * a));
  *vdw = 1.0e-4f * v / (a * a);
}
static void cutoff_fn(double rij, double* fc, double* dfc) {
  double t = tanh(BO_ALFA * (rij - BO_R0));
  *dfc = -0.5f * BO_ALFA * (1.0f - t * t);
  *fc = 0.5f * (1.0f - t);
}

/* ---- list settings: cpu/cpumd/Host.cpp:57-61 ---- */
void orc_list_settings(float rs, float rcut, float* maxnlmove, float* maxnlmovesq,
                       float* rcutsq) {
  *maxnlmove = (rs - rcut) * 0.5f;
  *maxnlmovesq = (float)pow((double)*maxnlmove, 2);
  *rcutsq = (float)pow((double)rcut, 2);
}

/* ---- cpu/cpumd/Host.cpp:245-271 readyList ---- */
void orc_ready_list(const double* pos4, const double* vel3, int n, double* vmax,
                    double* box) {
  double hv = 0, bs = 0;
  for (int i = 0; i < n; i++) {
    const double* v = vel3 + 3 * i;
    double s = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (s > hv) hv = s;
    for (int d = 0; d < 3; d++)
      if (bs < fabs(pos4[4 * i + d])) bs = fabs(pos4[4 * i + d]);
  }
  *vmax = hv;
  *box = bs * 2;
}

/* ---- cpu/cpumd/Host.cpp:289-290; vmax = 0 or an out-of-range quotient
 * means "never again" (the reference's (int) cast is undefined there) ---- */
int orc_next_build(float maxnlmove, double vmax, double dt, int t) {
  double q = ((double)maxnlmove / vmax) / fabs(dt);
  if (!(q < 2147483647.0) || q != q) return INT_MAX;
  long long nb = (long long)(int)q + t;
  return nb > INT_MAX ? INT_MAX : (int)nb;
}

/* ---- neighbour list: common/NeighborList.cpp:14-156 ---- */
typedef struct {
  int64_t* key;
  int* id;
  uint64_t mask;
} cell_table;

static int64_t cell_key(int cx, int cy, int cz) {
  return ((int64_t)(cx + 1) << 42) | ((int64_t)(cy + 1) << 21) | (int64_t)(cz + 1);
}
static uint64_t mix64(uint64_t x) {
  x ^= x >> 31;
  x *= 0x9e3779b97f4a7c15ULL;
  x ^= x >> 29;
  return x;
}
static int table_find(const cell_table* t, int64_t k) {
  uint64_t h = mix64((uint64_t)k) & t->mask;
  while (t->key[h] != -1) {
    if (t->key[h] == k) return t->id[h];
    h = (h + 1) & t->mask;
  }
  return -1;
}
static int table_insert(cell_table* t, int64_t k, int next_id) {
  uint64_t h = mix64((uint64_t)k) & t->mask;
  while (t->key[h] != -1) {
    if (t->key[h] == k) return t->id[h];
    h = (h + 1) & t->mask;
  }
  t->key[h] = k;
  t->id[h] = next_id;
  return next_id;
}

static void wrap_coord(double* x, double L) {
  /* periodic extension: x - L*floor((x + L/2)/L) */
  double h = L * 0.5;
  double q = floor((*x + h) / L);
  *x = *x - q * L;
}

orc_list* orc_build_list(double* pos4, int n, float rs, double box, int periodic) {
  orc_list* l = (orc_list*)calloc(1, sizeof(orc_list));
  if (!l) return NULL;
  l->n = n;
  l->periodic = periodic;
  l->box = box;
  int cells;
  double npos, cs;
  if (!periodic) {
    cells = (int)((box / (double)rs) + 0.99f);
    if (cells < 1) cells = 1;
    npos = box / 2;
    cs = (double)rs;
  } else {
    if (!(box > 2.0 * (double)rs)) {
      free(l);
      return NULL;
    }
    for (int i = 0; i < n; i++)
      for (int d = 0; d < 3; d++) wrap_coord(&pos4[4 * i + d], box);
    cells = (int)floor(box / (double)rs);
    if (cells < 3) cells = 1;
    npos = box * 0.5;
    cs = box / cells;
  }
  l->cells = cells;
  l->cell = (int*)malloc(sizeof(int) * 3 * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      int c = (int)((pos4[4 * i + d] + npos) / cs);
      if (periodic) {
        if (c >= cells) c = cells - 1;
        if (c < 0) c = 0;
      }
      l->cell[3 * i + d] = c;
    }
  /* group atoms by cell, ascending atom index inside a cell */
  uint64_t cap = 16;
  while (cap < 2 * (uint64_t)n + 16) cap <<= 1;
  cell_table t;
  t.key = (int64_t*)malloc(sizeof(int64_t) * cap);
  t.id = (int*)malloc(sizeof(int) * cap);
  t.mask = cap - 1;
  for (uint64_t k = 0; k < cap; k++) t.key[k] = -1;
  int* atom_cell = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int ncell = 0;
  for (int i = 0; i < n; i++) {
    int64_t k = cell_key(l->cell[3 * i], l->cell[3 * i + 1], l->cell[3 * i + 2]);
    int id = table_insert(&t, k, ncell);
    if (id == ncell) ncell++;
    atom_cell[i] = id;
  }
  int* cnt = (int*)calloc((size_t)ncell + 1, sizeof(int));
  int* start = (int*)calloc((size_t)ncell + 1, sizeof(int));
  for (int i = 0; i < n; i++) cnt[atom_cell[i]]++;
  int maxcell = 0;
  for (int c = 0; c < ncell; c++) {
    start[c + 1] = start[c] + cnt[c];
    if (cnt[c] > maxcell) maxcell = cnt[c];
  }
  int* member = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int* fill = (int*)calloc((size_t)ncell + 1, sizeof(int));
  for (int i = 0; i < n; i++) {
    int c = atom_cell[i];
    member[start[c] + fill[c]++] = i;
  }
  l->maxcell = maxcell;
  long long nls = (long long)maxcell * 27;
  if (nls > n - 1) nls = n - 1;
  if (nls < 0) nls = 0;
  l->nlistsize = (int)nls;
  size_t total = (size_t)nls * (size_t)n;
  l->rows = (int*)malloc(sizeof(int) * (total ? total : 1));
  l->code = (signed char*)malloc(total ? total : 1);
  int largest = 0;
  const int single = periodic && cells == 1;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : largest)
  for (int i = 0; i < n; i++) {
    int count = 0;
    int* row = l->rows + (size_t)i * nls;
    signed char* code = l->code + (size_t)i * nls;
    int cx = l->cell[3 * i], cy = l->cell[3 * i + 1], cz = l->cell[3 * i + 2];
    if (single) {
      for (int m = 0; m < n; m++) {
        if (m == i) continue;
        int im[3];
        for (int d = 0; d < 3; d++) {
          double dd = pos4[4 * i + d] - pos4[4 * m + d];
          im[d] = dd > 0.5 * box ? 1 : (dd < -0.5 * box ? -1 : 0);
        }
        row[count] = m;
        code[count] = (signed char)((im[0] + 1) * 9 + (im[1] + 1) * 3 + (im[2] + 1));
        count++;
      }
    } else {
      for (int dx = -1; dx < 2; dx++)
        for (int dy = -1; dy < 2; dy++)
          for (int dz = -1; dz < 2; dz++) {
            int nc[3] = {cx + dx, cy + dy, cz + dz};
            int im[3] = {0, 0, 0};
            int out = 0;
            for (int d = 0; d < 3; d++) {
              if (!periodic) {
                if (nc[d] >= cells || nc[d] < 0) out = 1;
              } else {
                if (nc[d] < 0) { nc[d] += cells; im[d] = -1; }
                if (nc[d] >= cells) { nc[d] -= cells; im[d] = 1; }
              }
            }
            if (out) continue;
            int c = table_find(&t, cell_key(nc[0], nc[1], nc[2]));
            if (c < 0) continue;
            signed char cd = (signed char)((im[0] + 1) * 9 + (im[1] + 1) * 3 + (im[2] + 1));
            for (int k = start[c]; k < start[c + 1]; k++) {
              int m = member[k];
              if (m == i) continue;
              row[count] = m;
              code[count] = cd;
              count++;
            }
          }
    }
    if (count > largest) largest = count;
    for (int k = count; k < nls; k++) {
      row[k] = -1;
      code[k] = 13;
    }
  }
  l->nlargest = largest;
  free(t.key);
  free(t.id);
  free(atom_cell);
  free(cnt);
  free(start);
  free(member);
  free(fill);
  return l;
}

void orc_free_list(orc_list* l) {
  if (!l) return;
  free(l->rows);
  free(l->code);
  free(l->cell);
  free(l);
}

/* position of list entry k of row i, with its periodic image applied */
static void entry_pos(const double* pos4, const orc_list* l, int j, signed char code,
                      double* p) {
  p[0] = pos4[4 * j];
  p[1] = pos4[4 * j + 1];
  p[2] = pos4[4 * j + 2];
  if (l->periodic && code != 13) {
    int ix = code / 9 - 1, iy = (code / 3) % 3 - 1, iz = code % 3 - 1;
    p[0] = p[0] + (double)ix * l->box;
    p[1] = p[1] + (double)iy * l->box;
    p[2] = p[2] + (double)iz * l->box;
  }
}

/* ---- cpu/common/Device.cpp:17-39 predict ---- */
void orc_predict(double* r4, double* v3, double* a3, double* b3, double* c3, double dt,
                 int nop) {
  double c1 = dt;
  double c2 = c1 * dt / 2.0f;
  double c3_ = c2 * dt / 3.0f;
  double c4 = c3_ * dt / 4.0f;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nop; i++) {
    double* r = r4 + 4 * i;
    double* v = v3 + 3 * i;
    double* a = a3 + 3 * i;
    double* b = b3 + 3 * i;
    double* c = c3 + 3 * i;
    for (int d = 0; d < 3; d++) r[d] = r[d] + c1 * v[d] + c2 * a[d] + c3_ * b[d] + c4 * c[d];
    for (int d = 0; d < 3; d++) v[d] = v[d] + c1 * a[d] + c2 * b[d] + c3_ * c[d];
    for (int d = 0; d < 3; d++) a[d] = a[d] + c1 * b[d] + c2 * c[d];
    for (int d = 0; d < 3; d++) b[d] = b[d] + c1 * c[d];
  }
}

/* ---- cpu/common/Device.cpp:44-120 correct (walls optional) ---- */
void orc_correct(double* r4, double* v3, const double* f3, double* a3, double* b3,
                 double* c3, double dt, int nop, double npos, int* flag, float energy_loss,
                 int walls, const orc_species* sp) {
  double c1 = dt;
  double c2 = c1 * dt / 2.0f;
  double c3_ = c2 * dt / 3.0f;
  double c4 = c3_ * dt / 4.0f;
  double cr = GEAR1 * c2;
  double cv = GEAR2 * c2 / c1;
  double cb = GEAR3 * c2 / c3_;
  double cc = GEAR4 * c2 / c4;
  int hit = 0;
#pragma omp parallel for schedule(static) reduction(| : hit)
  for (int i = 0; i < nop; i++) {
    double* r = r4 + 4 * i;
    double* v = v3 + 3 * i;
    const double* f = f3 + 3 * i;
    double* a = a3 + 3 * i;
    double* b = b3 + 3 * i;
    double* c = c3 + 3 * i;
    double mass = get_mass((int)r[3], sp);
    double ai[3], corr[3];
    for (int d = 0; d < 3; d++) ai[d] = f[d] / mass;
    for (int d = 0; d < 3; d++) corr[d] = ai[d] - a[d];
    for (int d = 0; d < 3; d++) r[d] = r[d] + cr * corr[d];
    for (int d = 0; d < 3; d++) v[d] = v[d] + cv * corr[d];
    for (int d = 0; d < 3; d++) a[d] = ai[d];
    for (int d = 0; d < 3; d++) b[d] = b[d] + cb * corr[d];
    for (int d = 0; d < 3; d++) c[d] = c[d] + cc * corr[d];
    if (!walls) continue;
    if (r[0] > npos && r[1] > 0) { hit = 1; v[0] = -v[0] * energy_loss; r[0] = npos; }
    if (r[0] > npos && r[1] < 0) { hit = 1; r[0] = -npos; }
    if (r[0] < -npos) { hit = 1; v[0] = -v[0]; r[0] = -npos; }
    if (fabs(r[1]) > npos) { hit = 1; v[1] = -v[1]; r[1] = npos * (r[1] / fabs(r[1])); }
    if (fabs(r[2]) > npos) { hit = 1; v[2] = -v[2]; r[2] = npos * (r[2] / fabs(r[2])); }
  }
  *flag = hit;
}

/* ---- cpu/common/Device.cpp:125-133 calculateAccelerations ---- */
void orc_accelerations(const double* pos4, double* a3, const double* f3, int n,
                       const orc_species* sp) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    double mass = get_mass((int)pos4[4 * i + 3], sp);
    for (int d = 0; d < 3; d++) a3[3 * i + d] = f3[3 * i + d] / mass;
  }
}

/* ---- LJ: cpu/common/LennardJones.h:12-30 (pair) and :35-93 (loop) ---- */
static void lj_select(int ti, int tj, const orc_species* sp, double* sig, double* eps) {
  int select = (ti == SP_NG) ? tj : ti;
  if (select == SP_N) {
    *eps = sp->epsNGN;
    *sig = sp->sigNGN;
  } else if (select == SP_O) {
    *eps = sp->epsNGO;
    *sig = sp->sigNGO;
  } else {
    *eps = sp->epsNG;
    *sig = sp->sigNG;
  }
}

void orc_lj_forces(const double* pos4, double* f3, int n, const orc_list* l,
                   double rcutsq, const orc_species* sp, double* energy) {
  const int nls = l->nlistsize, nlargest = l->nlargest;
  double e_sum = 0, es_sum = 0, w_sum = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : e_sum, es_sum, w_sum)
  for (int i = 0; i < n; i++) {
    double fx = 0.0, fy = 0.0, fz = 0.0, ei = 0, esi = 0, wi = 0;
    const double* pi = pos4 + 4 * i;
    int itype = (int)pi[3];
    const int* row = l->rows + (size_t)i * nls;
    const signed char* code = l->code + (size_t)i * nls;
    for (int j = 0; j < nlargest && row[j] != -1; j++) {
      int jp = row[j];
      double pj[3];
      entry_pos(pos4, l, jp, code[j], pj);
      double ijx = pi[0] - pj[0], ijy = pi[1] - pj[1], ijz = pi[2] - pj[2];
      double rij = ijx * ijx + ijy * ijy + ijz * ijz;
      if (rij >= rcutsq) continue;
      double r2 = rij;
      rij = sqrt(rij);
      int jtype = (int)pos4[4 * jp + 3];
      if (jtype == SP_NG || itype == SP_NG) {
        double sig, eps;
        lj_select(itype, jtype, sp, &sig, &eps);
        double sigsq = sig * sig;
        double con = 24.0f * eps / sigsq;
        double dist2 = rij * rij;
        dist2 /= sigsq;
        double dist4 = dist2 * dist2;
        double dist8 = dist4 * dist4;
        double dist14 = dist2 * dist4 * dist8;
        double invdist8 = 1.0f / dist8;
        double invdist14 = 1.0f / dist14;
        double s = (2 * invdist14) - invdist8;
        double fij = s * con;
        fx += ijx * fij;
        fy += ijy * fij;
        fz += ijz * fij;
        if (energy) {
          double sr2 = sig * sig / r2;
          double sr6 = sr2 * sr2 * sr2;
          double e = 2.0f * eps * (sr6 * sr6 - sr6);
          double src2 = sig * sig / rcutsq;
          double src6 = src2 * src2 * src2;
          ei += e;
          esi += e - 2.0f * eps * (src6 * src6 - src6);
          wi += 0.5 * (ijx * (ijx * fij) + ijy * (ijy * fij) + ijz * (ijz * fij));
        }
      }
    }
    f3[3 * i] = fx;
    f3[3 * i + 1] = fy;
    f3[3 * i + 2] = fz;
    e_sum += ei;
    es_sum += esi;
    w_sum += wi;
  }
  if (energy) {
    energy[0] = e_sum;
    energy[1] = es_sum;
    energy[2] = w_sum;
  }
}

/* ---- bond order: cpu/common/BondOrderFuncs.h ---- */
typedef struct {
  const double* pos4;
  const orc_list* l;
  double rcutsq;
  double* xsi; /* per (i, slot) */
  double* xsj;
  unsigned char* xw; /* written flag */
} mb_ctx;

/* BondOrderFuncs.h:12-143 bondOrder1.  pi, pj: positions of i and of j's
 * image; slot: j's slot in row i (xi is stored there). */
static void bond_order1(const mb_ctx* c, double re, double rij, int i, int j, int slot,
                        const double* pi, const double* pj, const double* ij, double* bo,
                        double* dbo) {
  const orc_list* l = c->l;
  const int nls = l->nlistsize, nlargest = l->nlargest;
  double drijx = (ij[0]) / rij, drijy = (ij[1]) / rij, drijz = (ij[2]) / rij;
  double xsi = 0, xsj = 0;
  double dxsix = 0.0f, dxsiy = 0.0f, dxsiz = 0.0f;
  double dxsjx = 0.0f, dxsjy = 0.0f, dxsjz = 0.0f;
  const int* row = l->rows + (size_t)i * nls;
  const signed char* code = l->code + (size_t)i * nls;
  const double E = exp(BO_LAMDA3 * (rij - re));
  for (int m = 0; m < nlargest && row[m] != -1; m++) {
    int mp = row[m];
    int mtype = (int)c->pos4[4 * mp + 3];
    if (mtype == SP_NG) continue;
    if (mp == j) continue;
    double pm[3];
    entry_pos(c->pos4, l, mp, code[m], pm);
    double imx = pi[0] - pm[0], imy = pi[1] - pm[1], imz = pi[2] - pm[2];
    double rim = imx * imx + imy * imy + imz * imz;
    if (rim >= c->rcutsq) continue;
    rim = sqrt(rim);
    double jmx = pj[0] - pm[0], jmy = pj[1] - pm[1], jmz = pj[2] - pm[2];
    double rjm = sqrt(jmx * jmx + jmy * jmy + jmz * jmz);
    double fci, dfci, fcj, dfcj;
    cutoff_fn(rim, &fci, &dfci);
    cutoff_fn(rjm, &fcj, &dfcj);
    double drimx = (pi[0] - pm[0]) / rim;
    double drimy = (pi[1] - pm[1]) / rim;
    double drimz = (pi[2] - pm[2]) / rim;
    if (fci > 0) {
      double icosthe = (rij * rij + rim * rim - rjm * rjm) / (2.0f * rij * rim);
      double hc = BO_H - icosthe;
      double q = BO_D + hc * hc;
      double igthe = 1.0f + BO_C / BO_D - BO_C / q;
      xsi += fci * igthe * E;
      double num2 = (rij * rij + rim * rim - rjm * rjm);
      double den = (4.0f * rij * rij * rim * rim);
      double dcx = ((2.0f * rij * drijx + 2.0f * rim * drimx) * 2.0f * rij * rim -
                    (2.0f * rim * drijx + 2.0f * rij * drimx) * num2) / den;
      double dcy = ((2.0f * rij * drijy + 2.0f * rim * drimy) * 2.0f * rij * rim -
                    (2.0f * rim * drijy + 2.0f * rij * drimy) * num2) / den;
      double dcz = ((2.0f * rij * drijz + 2.0f * rim * drimz) * 2.0f * rij * rim -
                    (2.0f * rim * drijz + 2.0f * rij * drimz) * num2) / den;
      double gpre = -BO_C / (q * q) * 2.0f * hc;
      double dgx = gpre * dcx, dgy = gpre * dcy, dgz = gpre * dcz;
      dxsix += (dfci * drimx * igthe * E + fci * dgx * E + fci * igthe * BO_LAMDA3 * E * drijx);
      dxsiy += (dfci * drimy * igthe * E + fci * dgy * E + fci * igthe * BO_LAMDA3 * E * drijy);
      dxsiz += (dfci * drimz * igthe * E + fci * dgz * E + fci * igthe * BO_LAMDA3 * E * drijz);
    }
    if (fcj > 0) {
      double jcosthe = (rij * rij + rjm * rjm - rim * rim) / (2.0f * rij * rjm);
      double hc = BO_H - jcosthe;
      double q = BO_D + hc * hc;
      double jgthe = 1.0f + BO_C / BO_D - BO_C / q;
      xsj += fcj * jgthe * E;
      double num2 = (rij * rij + rjm * rjm - rim * rim);
      double den = (4.0f * rij * rij * rjm * rjm);
      double dcx = ((2.0f * rij * drijx - 2.0f * rim * drimx) * 2.0f * rij * rjm -
                    2.0f * rjm * drijx * num2) / den;
      double dcy = ((2.0f * rij * drijy - 2.0f * rim * drimy) * 2.0f * rij * rjm -
                    2.0f * rjm * drijy * num2) / den;
      double dcz = ((2.0f * rij * drijz - 2.0f * rim * drimz) * 2.0f * rij * rjm -
                    2.0f * rjm * drijz * num2) / den;
      double gpre = -BO_C / (q * q) * 2.0f * hc;
      double dgx = gpre * dcx, dgy = gpre * dcy, dgz = gpre * dcz;
      dxsjx += (fcj * (dgx * E + BO_LAMDA3 * E * drijx * jgthe));
      dxsjy += (fcj * (dgy * E + BO_LAMDA3 * E * drijy * jgthe));
      dxsjz += (fcj * (dgz * E + BO_LAMDA3 * E * drijz * jgthe));
    }
  }
  size_t s = (size_t)i * nls + slot;
  c->xsi[s] = xsi;
  c->xsj[s] = xsj;
  c->xw[s] = 1;
  double bij = 1.0f / (1.0f + xsi);
  double pbi = (1.0f / ((1.0f + xsi) * (1.0f + xsi)));
  double bji = 1.0f / (1.0f + xsj);
  double pbj = (1.0f / ((1.0f + xsj) * (1.0f + xsj)));
  *bo = 0.5f * (bij + bji);
  dbo[0] = 0.5f * (pbi * dxsix + pbj * dxsjx);
  dbo[1] = 0.5f * (pbi * dxsiy + pbj * dxsjy);
  dbo[2] = 0.5f * (pbi * dxsiz + pbj * dxsjz);
}

/* BondOrderFuncs.h:148-237 bondOrder2 (k third body of pair i,j); pk, pi, pj
 * are the positions of k and of the images of i and j seen from k. */
static void bond_order2(double re, double rij, double rik, const double* pk,
                        const double* pi, const double* pj, double xsi, double xsj,
                        double* dbo) {
  dbo[0] = dbo[1] = dbo[2] = 0;
  double jkx = pj[0] - pk[0], jky = pj[1] - pk[1], jkz = pj[2] - pk[2];
  double rjk = sqrt(jkx * jkx + jky * jky + jkz * jkz);
  double drjkx = (pk[0] - pj[0]) / rjk, drjky = (pk[1] - pj[1]) / rjk,
         drjkz = (pk[2] - pj[2]) / rjk;
  double drikx = (pk[0] - pi[0]) / rik, driky = (pk[1] - pi[1]) / rik,
         drikz = (pk[2] - pi[2]) / rik;
  double fci, dfci, fcj, dfcj;
  cutoff_fn(rik, &fci, &dfci);
  cutoff_fn(rjk, &fcj, &dfcj);
  const double E = exp(BO_LAMDA3 * (rij - re));
  if (fci > 0) {
    double icosthe = (rij * rij + rik * rik - rjk * rjk) / (2.0f * rij * rik);
    double hc = BO_H - icosthe;
    double q = BO_D + hc * hc;
    double igthe = 1.0f + BO_C / BO_D - BO_C / q;
    double num2 = (rij * rij + rik * rik - rjk * rjk);
    double den = (4.0f * rij * rij * rik * rik);
    double dcx = ((2.0f * rik * drikx - 2.0f * rjk * drjkx) * 2.0f * rij * rik - (2.0f * rij * drikx) * num2) / den;
    double dcy = ((2.0f * rik * driky - 2.0f * rjk * drjky) * 2.0f * rij * rik - (2.0f * rij * driky) * num2) / den;
    double dcz = ((2.0f * rik * drikz - 2.0f * rjk * drjkz) * 2.0f * rij * rik - (2.0f * rij * drikz) * num2) / den;
    double gpre = -BO_C / (q * q) * 2.0f * hc;
    double idxsix = dfci * drikx * igthe * E + fci * (gpre * dcx) * E;
    double idxsiy = dfci * driky * igthe * E + fci * (gpre * dcy) * E;
    double idxsiz = dfci * drikz * igthe * E + fci * (gpre * dcz) * E;
    double p = (1.0f / ((1.0f + xsi) * (1.0f + xsi)));
    dbo[0] += (0.5f * (p * idxsix));
    dbo[1] += (0.5f * (p * idxsiy));
    dbo[2] += (0.5f * (p * idxsiz));
  }
  if (fcj > 0) {
    double jcosthe = (rij * rij + rjk * rjk - rik * rik) / (2.0f * rij * rjk);
    double hc = BO_H - jcosthe;
    double q = BO_D + hc * hc;
    double jgthe = 1.0f + BO_C / BO_D - BO_C / q;
    double num2 = (rij * rij + rjk * rjk - rik * rik);
    double den = (4.0f * rij * rij * rjk * rjk);
    double dcx = ((2.0f * rjk * drjkx - 2.0f * rik * drikx) * 2.0f * rij * rjk - (2.0f * rij * drjkx) * num2) / den;
    double dcy = ((2.0f * rjk * drjky - 2.0f * rik * driky) * 2.0f * rij * rjk - (2.0f * rij * drjky) * num2) / den;
    double dcz = ((2.0f * rjk * drjkz - 2.0f * rik * drikz) * 2.0f * rij * rjk - (2.0f * rij * drjkz) * num2) / den;
    double gpre = -BO_C / (q * q) * 2.0f * hc;
    double jdxsix = dfcj * drjkx * jgthe * E + fcj * (gpre * dcx) * E;
    double jdxsiy = dfcj * drjky * jgthe * E + fcj * (gpre * dcy) * E;
    double jdxsiz = dfcj * drjkz * jgthe * E + fcj * (gpre * dcz) * E;
    double p = (1.0f / ((1.0f + xsj) * (1.0f + xsj)));
    dbo[0] += (0.5f * (p * jdxsix));
    dbo[1] += (0.5f * (p * jdxsiy));
    dbo[2] += (0.5f * (p * jdxsiz));
  }
}

/* BondOrderFuncs.h:283-397 manyBodyForces */
void orc_mb_forces(const double* pos4, double* f3, int mbp, const orc_list* l,
                   double rcutsq, int ljexist, long long* missing, double* energy) {
  const int nls = l->nlistsize, nlargest = l->nlargest;
  size_t tot = (size_t)mbp * nls;
  mb_ctx c;
  c.pos4 = pos4;
  c.l = l;
  c.rcutsq = rcutsq;
  c.xsi = (double*)malloc(sizeof(double) * (tot ? tot : 1));
  c.xsj = (double*)malloc(sizeof(double) * (tot ? tot : 1));
  c.xw = (unsigned char*)calloc(tot ? tot : 1, 1);
  const double cut_rijsq = CUTOFF_RIJSQ;
  double e_sum = 0, w_sum = 0;
  double* fmb1 = energy ? (double*)malloc(sizeof(double) * 3 * (size_t)(mbp ? mbp : 1)) : NULL;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : e_sum)
  for (int i = 0; i < mbp; i++) {
    const double* pi = pos4 + 4 * i;
    int type = (int)pi[3];
    double fx = 0.0, fy = 0.0, fz = 0.0, ei = 0;
    const int* row = l->rows + (size_t)i * nls;
    const signed char* code = l->code + (size_t)i * nls;
    for (int j = 0; j < nlargest && row[j] != -1; j++) {
      int jp = row[j];
      double pj[3];
      entry_pos(pos4, l, jp, code[j], pj);
      double ij[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
      double rij = ij[0] * ij[0] + ij[1] * ij[1] + ij[2] * ij[2];
      if (rij >= rcutsq || rij > cut_rijsq) continue;
      rij = sqrt(rij);
      int jtype = (int)pos4[4 * jp + 3];
      if (jtype == SP_NG) continue;
      /* BondOrderFuncs.h:242-278 bondForces */
      double va = 0, dva = 0, vr = 0, dvr = 0, vdw, dvdw, bo = 0;
      double dbo[3] = {0.0f, 0.0f, 0.0f};
      double fcut, dfcut;
      cutoff_fn(rij / 10, &fcut, &dfcut);
      if (fcut > 0) {
        double de = get_de(type, jtype), re = get_re(type, jtype), beta = get_beta(type, jtype);
        attractive(&va, &dva, rij, de, beta, re);
        repulsive(&vr, &dvr, rij, de, beta, re);
        bond_order1(&c, re, rij, i, jp, j, pi, pj, ij, &bo, dbo);
      }
      vander_waals(&vdw, &dvdw, rij, get_r0v(type, jtype));
      double fij = dvr - bo * dva + dvdw;
      fx += fij * (ij[0]) / rij - dbo[0] * va;
      fy += fij * (ij[1]) / rij - dbo[1] * va;
      fz += fij * (ij[2]) / rij - dbo[2] * va;
      ei += 0.5f * ((vr - bo * va) + vdw);
    }
    if (fmb1) {
      fmb1[3 * i] = fx;
      fmb1[3 * i + 1] = fy;
      fmb1[3 * i + 2] = fz;
    }
    if (ljexist) {
      f3[3 * i] += fx;
      f3[3 * i + 1] += fy;
      f3[3 * i + 2] += fz;
    } else {
      f3[3 * i] = fx;
      f3[3 * i + 1] = fy;
      f3[3 * i + 2] = fz;
    }
    e_sum += ei;
  }
  /* pass 2, BondOrderFuncs.h:339-393; W_mb = sum_i r_i . F_i(mb) needs the
   * bond-order parts alone, kept in fmb1 (pass 1) and fmb (pass 2) */
  double* fmb = energy ? (double*)malloc(sizeof(double) * 3 * (size_t)(mbp ? mbp : 1)) : NULL;
  long long miss = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : miss)
  for (int k = 0; k < mbp; k++) {
    const double* pk = pos4 + 4 * k;
    const int* row = l->rows + (size_t)k * nls;
    const signed char* code = l->code + (size_t)k * nls;
    double f2x = 0, f2y = 0, f2z = 0;
    double fk[3] = {f3[3 * k], f3[3 * k + 1], f3[3 * k + 2]};
    for (int ii = 0; ii < nlargest && row[ii] != -1; ii++) {
      int ip = row[ii];
      int itype = (int)pos4[4 * ip + 3];
      double pi[3];
      entry_pos(pos4, l, ip, code[ii], pi);
      double ikx = pk[0] - pi[0], iky = pk[1] - pi[1], ikz = pk[2] - pi[2];
      double rik = ikx * ikx + iky * iky + ikz * ikz;
      if (rik >= rcutsq) continue;
      rik = sqrt(rik);
      const int* rowi = l->rows + (size_t)ip * nls;
      for (int jj = 0; jj < nlargest && row[jj] != -1; jj++) {
        int jp = row[jj];
        int jtype = (int)pos4[4 * jp + 3];
        if (ip == jp) continue;
        double pj[3];
        entry_pos(pos4, l, jp, code[jj], pj);
        double ijx = pi[0] - pj[0], ijy = pi[1] - pj[1], ijz = pi[2] - pj[2];
        double rij = ijx * ijx + ijy * ijy + ijz * ijz;
        if (rij >= rcutsq || rij > cut_rijsq) continue;
        rij = sqrt(rij);
        double de = get_de(itype, jtype), re = get_re(itype, jtype), beta = get_beta(itype, jtype);
        double va, dva, dbo[3];
        attractive(&va, &dva, rij, de, beta, re);
        /* xi(ip, jp): find jp's slot in row ip */
        double xsi = 0, xsj = 0;
        int found = 0;
        if (ip < mbp) {
          for (int s = 0; s < nlargest && rowi[s] != -1; s++)
            if (rowi[s] == jp) {
              size_t q = (size_t)ip * nls + s;
              if (c.xw[q]) {
                xsi = c.xsi[q];
                xsj = c.xsj[q];
                found = 1;
              }
              break;
            }
        }
        if (!found) miss++;
        bond_order2(re, rij, rik, pk, pi, pj, xsi, xsj, dbo);
        fk[0] -= 0.5f * dbo[0] * va;
        fk[1] -= 0.5f * dbo[1] * va;
        fk[2] -= 0.5f * dbo[2] * va;
        f2x -= 0.5f * dbo[0] * va;
        f2y -= 0.5f * dbo[1] * va;
        f2z -= 0.5f * dbo[2] * va;
      }
    }
    f3[3 * k] = fk[0];
    f3[3 * k + 1] = fk[1];
    f3[3 * k + 2] = fk[2];
    if (fmb) {
      fmb[3 * k] = f2x;
      fmb[3 * k + 1] = f2y;
      fmb[3 * k + 2] = f2z;
    }
  }
  if (energy) {
    for (int i = 0; i < mbp; i++)
      for (int d = 0; d < 3; d++) w_sum += pos4[4 * i + d] * (fmb1[3 * i + d] + fmb[3 * i + d]);
    energy[0] = e_sum;
    energy[1] = w_sum;
    free(fmb);
    free(fmb1);
  }
  if (missing) *missing = miss;
  free(c.xsi);
  free(c.xsj);
  free(c.xw);
}

/* ---- common/DebugCalculations.cpp:46-124 PerformCalculations ---- */
void orc_perform_calculations(const double* pos4, const double* vel3, int n, double* out,
                              const orc_species* sp) {
  double mass = 0, cmvx = 0, cmvy = 0, cmvz = 0, total = 0;
  double ke = 0, temp = 0, cx = 0, cy = 0, cz = 0;
  for (int i = 0; i < n; i++) {
    mass = get_mass((int)pos4[4 * i + 3], sp);
    const double* v = vel3 + 3 * i;
    ke += mass * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    cmvx += mass * v[0];
    cmvy += mass * v[1];
    cmvz += mass * v[2];
    total += mass;
    cx += mass * pos4[4 * i];
    cy += mass * pos4[4 * i + 1];
    cz += mass * pos4[4 * i + 2];
  }
  cx /= total;
  cy /= total;
  cz /= total;
  out[4] = cmvx;
  out[5] = cmvy;
  out[6] = cmvz;
  cmvx /= total;
  cmvy /= total;
  cmvz /= total;
  for (int i = 0; i < n; i++) {
    mass = get_mass((int)pos4[4 * i + 3], sp);
    const double* v = vel3 + 3 * i;
    temp += mass * ((v[0] - cmvx) * (v[0] - cmvx) + (v[1] - cmvy) * (v[1] - cmvy) +
                    (v[2] - cmvz) * (v[2] - cmvz));
  }
  temp /= (3.0f * ((double)n) * KB_FLOAT);
  ke /= 2;
  out[0] = cx;
  out[1] = cy;
  out[2] = cz;
  out[3] = ke;
  out[7] = temp;
}

/* ---- common/DebugCalculations.cpp:129-270 calculatePotentional ---- */
void orc_calculate_potential(const double* pos4, int n, double* vib_lj, double* vib_mb,
                             const orc_species* sp) {
  double elj = 0, emb = 0;
  for (int i = 0; i < n; i++) {
    int itype = (int)pos4[4 * i + 3];
    for (int j = 0; j < n; j++) {
      if (i == j) continue;
      int jtype = (int)pos4[4 * j + 3];
      double ijx = pos4[4 * i] - pos4[4 * j];
      double ijy = pos4[4 * i + 1] - pos4[4 * j + 1];
      double ijz = pos4[4 * i + 2] - pos4[4 * j + 2];
      double rijsq = ijx * ijx + ijy * ijy + ijz * ijz;
      if (jtype == SP_NG || itype == SP_NG) {
        double sig, eps;
        lj_select(itype, jtype, sp, &sig, &eps);
        double sr2 = sig * sig / rijsq;
        double sr6 = sr2 * sr2 * sr2;
        elj += 2.0f * eps * (sr6 * sr6 - sr6);
      } else {
        double va = 0, dva, vr = 0, dvr, vdw, dvdw;
        double rij = sqrt(rijsq);
        double bo = 0;
        if (rij > CUTOFF_RIJ) continue;
        double fcut, dfcut;
        cutoff_fn(rij / 10, &fcut, &dfcut);
        if (fcut > 0) {
          double de = get_de(itype, jtype), re = get_re(itype, jtype),
                 beta = get_beta(itype, jtype);
          attractive(&va, &dva, rij, de, beta, re);
          repulsive(&vr, &dvr, rij, de, beta, re);
          double xsi = 0, xsj = 0;
          for (int m = 0; m < n; m++) {
            int mtype = (int)pos4[4 * m + 3];
            if (mtype == SP_NG) continue;
            if (m == j || m == i) continue;
            double imx = pos4[4 * i] - pos4[4 * m];
            double imy = pos4[4 * i + 1] - pos4[4 * m + 1];
            double imz = pos4[4 * i + 2] - pos4[4 * m + 2];
            double rim = sqrt(imx * imx + imy * imy + imz * imz);
            double jmx = pos4[4 * j] - pos4[4 * m];
            double jmy = pos4[4 * j + 1] - pos4[4 * m + 1];
            double jmz = pos4[4 * j + 2] - pos4[4 * m + 2];
            double rjm = sqrt(jmx * jmx + jmy * jmy + jmz * jmz);
            double fci, dfci, fcj, dfcj;
            cutoff_fn(rim, &fci, &dfci);
            cutoff_fn(rjm, &fcj, &dfcj);
            if (fci > 0) {
              double icosthe = (rij * rij + rim * rim - rjm * rjm) / (2.0f * rij * rim);
              double igthe = 1.0f + BO_C / BO_D - BO_C / (BO_D + (BO_H - icosthe) * (BO_H - icosthe));
              xsi += fci * igthe * exp(BO_LAMDA3 * (rij - re));
            }
            if (fcj > 0) {
              double jcosthe = (rij * rij + rjm * rjm - rim * rim) / (2.0f * rij * rjm);
              double jgthe = 1.0f + BO_C / BO_D - BO_C / (BO_D + (BO_H - jcosthe) * (BO_H - jcosthe));
              xsj += fcj * jgthe * exp(BO_LAMDA3 * (rij - re));
            }
          }
          double bij = 1.0f / (1.0f + xsi);
          double bji = 1.0f / (1.0f + xsj);
          bo = 0.5f * (bij + bji);
        }
        vander_waals(&vdw, &dvdw, rij, get_r0v(itype, jtype));
        emb += 0.5f * ((vr - bo * va) + vdw);
      }
    }
  }
  *vib_lj = elj;
  *vib_mb = emb;
}

/* ---- one vxcm pass of cpu/cpumd/Host.cpp:hostMain ---- */
static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static void record(const orc_run_params* p, const orc_species* sp, double* pos4,
                   const double* vel3, const orc_list* ljl, const orc_list* mbl,
                   double lj_rcutsq, double mb_rcutsq, double* out) {
  int n = p->n_lj + p->n_mb;
  orc_perform_calculations(pos4, vel3, n, out, sp);
  double elj[3] = {0, 0, 0}, emb[2] = {0, 0};
  double* ftmp = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  if (p->use_lj && ljl) orc_lj_forces(pos4, ftmp, n, ljl, lj_rcutsq, sp, elj);
  if (p->use_mb && mbl) {
    memset(ftmp, 0, sizeof(double) * 3 * (size_t)n);
    orc_mb_forces(pos4, ftmp, p->n_mb, mbl, mb_rcutsq, 0, NULL, emb);
  }
  free(ftmp);
  out[8] = elj[0];
  out[9] = elj[1];
  out[10] = emb[0];
  out[11] = elj[2] + emb[1];
}

static void sync_schedule(const orc_run_params* p, int* lj_next, int* mb_next) {
  int m = INT_MAX;
  if (p->use_lj && *lj_next < m) m = *lj_next;
  if (p->use_mb && *mb_next < m) m = *mb_next;
  if (p->use_lj) *lj_next = m;
  if (p->use_mb) *mb_next = m;
}

int orc_run(const orc_run_params* p, double* pos4, double* vel3, double* acc3, double* b3,
            double* c3, double* f3, double* thermo, long long* stats, double* elapsed_ms) {
#ifdef _OPENMP
  if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
  orc_species sp;
  orc_species_get(p->species, &sp);
  int n = p->n_lj + p->n_mb;
  double boxSize = pow(n, 1.0 / 3.0) * 52.8;
  float lj_mv = 0, lj_mvsq = 0, lj_rc2 = 0, mb_mv = 0, mb_mvsq = 0, mb_rc2 = 0;
  if (p->use_lj) orc_list_settings(p->lj_rs, p->lj_rcut, &lj_mv, &lj_mvsq, &lj_rc2);
  if (p->use_mb) orc_list_settings(p->mb_rs, p->mb_rcut, &mb_mv, &mb_mvsq, &mb_rc2);
  float energy_loss = sqrtf(p->energy_loss);
  orc_list *ljl = NULL, *mbl = NULL;
  int t = 0, lj_next = 0, mb_next = 0, nrec = 0;
  long long builds = 0, hits = 0, missing = 0, miss1 = 0;
  double vmax, box_list;
  memset(acc3, 0, sizeof(double) * 3 * (size_t)n);
  memset(b3, 0, sizeof(double) * 3 * (size_t)n);
  memset(c3, 0, sizeof(double) * 3 * (size_t)n);
  for (int id = 0; id < n; id++) {
    double* r = pos4 + 4 * id;
    if (!p->periodic) {
      for (int d = 0; d < 3; d++)
        if (fabs(r[d]) > (boxSize / 2)) r[d] = (boxSize / 2) * (r[d] / fabs(r[d]));
    }
    vel3[3 * id] += p->vxcm;
  }
#define BUILD(which, lst, settings_mv, rs_, nn_, next_)                               \
  do {                                                                              \
    orc_free_list(lst);                                                             \
    lst = orc_build_list(pos4, nn_, rs_, p->periodic ? p->box : box_list, p->periodic); \
    if (!lst) return -1;                                                            \
    next_ = orc_next_build(settings_mv, vmax, p->dt, t);                           \
    builds++;                                                                       \
  } while (0)
  orc_ready_list(pos4, vel3, n, &vmax, &box_list);
  if (p->use_lj) BUILD(lj, ljl, lj_mv, p->lj_rs, n, lj_next);
  if (p->use_mb) BUILD(mb, mbl, mb_mv, p->mb_rs, p->n_mb, mb_next);
  if (p->periodic) sync_schedule(p, &lj_next, &mb_next);
  if (thermo) record(p, &sp, pos4, vel3, ljl, mbl, lj_rc2, mb_rc2, thermo + 12 * nrec++);
  double t0 = now_ms();
  if (p->use_lj) orc_lj_forces(pos4, f3, n, ljl, lj_rc2, &sp, NULL);
  if (p->use_mb) { orc_mb_forces(pos4, f3, p->n_mb, mbl, mb_rc2, p->use_lj, &miss1, NULL); missing += miss1; }
  orc_accelerations(pos4, acc3, f3, n, &sp);
  int printout = p->output_timesteps;
  while (t < p->timesteps) {
    if (lj_next == t || mb_next == t) {
      orc_ready_list(pos4, vel3, n, &vmax, &box_list);
      /* periodic box: positions are wrapped at a build, which would stale
       * the image codes of the other list, so both lists are rebuilt
       * together at the earlier of their two schedules */
      int due_lj = p->use_lj && lj_next == t, due_mb = p->use_mb && mb_next == t;
      if (p->periodic && (due_lj || due_mb)) {
        due_lj = p->use_lj;
        due_mb = p->use_mb;
      }
      if (due_lj) BUILD(lj, ljl, lj_mv, p->lj_rs, n, lj_next);
      if (due_mb) BUILD(mb, mbl, mb_mv, p->mb_rs, p->n_mb, mb_next);
      if (p->periodic) sync_schedule(p, &lj_next, &mb_next);
    }
    orc_predict(pos4, vel3, acc3, b3, c3, p->dt, n);
    if (p->use_lj) orc_lj_forces(pos4, f3, n, ljl, lj_rc2, &sp, NULL);
    if (p->use_mb) { orc_mb_forces(pos4, f3, p->n_mb, mbl, mb_rc2, p->use_lj, &miss1, NULL); missing += miss1; }
    int flag = 0;
    orc_correct(pos4, vel3, f3, acc3, b3, c3, p->dt, n, boxSize, &flag, energy_loss,
                !p->periodic, &sp);
    if (flag) {
      hits++;
      if (p->use_lj) orc_lj_forces(pos4, f3, n, ljl, lj_rc2, &sp, NULL);
      if (p->use_mb) { orc_mb_forces(pos4, f3, p->n_mb, mbl, mb_rc2, p->use_lj, &miss1, NULL); missing += miss1; }
      orc_accelerations(pos4, acc3, f3, n, &sp);
    }
    if (printout == t) {
      if (thermo) record(p, &sp, pos4, vel3, ljl, mbl, lj_rc2, mb_rc2, thermo + 12 * nrec++);
      printout += p->output_timesteps;
    }
    t++;
  }
#undef BUILD
  *elapsed_ms = now_ms() - t0;
  if (stats) {
    stats[0] = builds;
    stats[1] = hits;
    stats[2] = missing;
  }
  orc_free_list(ljl);
  orc_free_list(mbl);
  return nrec;
}

/* ---- equi: the reference's inverse error function and velocity draw ---- */

/* cpu/equi/Statistics.cpp:175-196 erf: the Taylor series for |x| <= 2.2 with
 * the reference's stopping test |term| / sum > 1e-12.  For x < 0 the sum is
 * negative, the test fails at once and the series stops after its first two
 * terms: the reference's erf, and so its inverf, is inaccurate for negative
 * arguments; that is kept.  Beyond 2.2, 1 - erfc(x). */
static double ref_erfc(double x);
static double ref_erf(double x) {
  const double two_sqrtpi = 1.128379167095512574;
  if (fabs(x) > 2.2) return 1.0 - ref_erfc(x);
  double sum = x, term = x, xsqr = x * x;
  int j = 1;
  do {
    term *= xsqr / j;
    sum -= term / (2 * j + 1);
    ++j;
    term *= xsqr / j;
    sum += term / (2 * j + 1);
    ++j;
  } while (fabs(term) / sum > 1e-12);
  return two_sqrtpi * sum;
}

/* Statistics.cpp:199-227 erfc: 1 - erf(x) for |x| < 2.2, 2 - erfc(-x) for
 * x < 0, else the continued fraction until two convergents agree to 1e-12. */
static double ref_erfc(double x) {
  const double one_sqrtpi = 0.564189583547756287;
  if (fabs(x) < 2.2) return 1.0 - ref_erf(x);
  if (x < 0) return 2.0 - ref_erfc(-x);
  double a = 1, b = x, c = x, d = x * x + 0.5, q1, q2 = b / d, nn = 1.0, t;
  do {
    t = a * nn + b * x;
    a = b;
    b = t;
    t = c * nn + d * x;
    c = d;
    d = t;
    nn += 0.5;
    q1 = q2;
    q2 = b / d;
  } while (fabs(q1 - q2) / q2 > 1e-12);
  return one_sqrtpi * exp(-x * x) * q2;
}

/* Statistics.cpp:25-41: second-order Newton steps on erf(x) - z from x = 0 */
static double inv_erf_small(double z) {
  const double c = 1.1283791670955125738961589; /* 2 / sqrt(pi) */
  double f = -z, f1 = c;
  double q = f / f1, x = -q, x0 = 0;
  while (fabs(x - x0) > 1e-12 && fabs(f) > 1e-14) {
    x0 = x;
    f = ref_erf(x) - z;
    f1 = c * exp(-x * x);
    q = f / f1;
    x -= q * (1 - x * q);
  }
  return x;
}

/* Statistics.cpp:58-64: the start value of inv_erfc_small */
static double lambert_w2(double z) {
  double logz = log(z);
  double slz = sqrt(logz);
  return slz - 0.25 * log(logz) / slz;
}

/* Statistics.cpp:74-95: Newton steps on erfc(sqrt(log(x))) - z */
static double inv_erfc_small(double z) {
  const double c = 1.7724538509055160272981675; /* sqrt(pi) */
  double f = 1, f1i = 0;
  double a = lambert_w2(1 / (c * z));
  double x = ref_erfc(a) / (c * a * z * z), x0 = 0;
  while (fabs(x - x0) > 1e-12 * x && fabs(f) > 1e-15 * z) {
    double slx;
    x0 = x;
    slx = sqrt(log(x));
    f = z - ref_erfc(slx);
    f1i = c * x * x * slx;
    x -= f * f1i * (1 - c * f * x * (slx + 0.25 / slx));
  }
  return sqrt(log(x));
}

/* cpu/equi/Statistics.cpp:115-140 inverf */
double orc_inverf(double z) {
  double az = fabs(z);
  if (az >= 1) {
    if (z == 1) return INFINITY;
    if (z == -1) return -INFINITY;
    return NAN;
  }
  if (az < 0.8125) return inv_erf_small(z);
  if (z > 0) return inv_erfc_small(1 - z);
  return -inv_erfc_small(z + 1);
}

/* cpu/equi/Host.cpp:416-572 chooseVelocities, with the uniforms y of
 * (rand() + 1) / MD_RANDMAX given (three per draw: x, y, z, in the
 * reference's order).  Many-body atoms i, i + 1 (i < n_mb) share one draw
 * made with atom i's mass, and the sums before the momentum removal count
 * such a pair once (:465-478); the z draw applies inverf before the affine
 * map (:457-461).  The removal loop (:480-515) is the reference's; where a
 * shift after the second does not shrink the largest momentum component (the
 * reference would loop forever) or max_shifts are spent, returns -1.  Returns the number of
 * uniforms used. */
long orc_choose_velocities(const double* pos4, double* vel3, int n, int n_mb, double temp,
                           int species, const double* u, long nu, long max_shifts,
                           long* shifts) {
  orc_species sp;
  orc_species_get(species, &sp);
  const double mass_of[3] = {sp.mN, sp.mO, sp.mNG};
  double cmvx = 0, cmvy = 0, cmvz = 0, totalm = 0, t = 0;
  long k = 0;
  for (int i = 0; i < n; i++) {
    double mass = mass_of[(int)pos4[4 * i + 3]];
    double y = k < nu ? u[k] : 0;
    k++;
    y = 2.0 * y - 1.0;
    y = orc_inverf(y);
    vel3[3 * i] = y * sqrt(2.0 * temp / mass);
    y = k < nu ? u[k] : 0;
    k++;
    y = 2.0 * y - 1.0;
    y = orc_inverf(y);
    vel3[3 * i + 1] = y * sqrt(2.0 * temp / mass);
    y = k < nu ? u[k] : 0;
    k++;
    y = orc_inverf(y);
    y = 2.0 * y - 1.0;
    vel3[3 * i + 2] = y * sqrt(2.0 * temp / mass);
    if (i < n_mb) {
      vel3[3 * (i + 1)] = vel3[3 * i];
      vel3[3 * (i + 1) + 1] = vel3[3 * i + 1];
      vel3[3 * (i + 1) + 2] = vel3[3 * i + 2];
      i++;
    }
    cmvx = cmvx + mass * vel3[3 * i];
    cmvy = cmvy + mass * vel3[3 * i + 1];
    cmvz = cmvz + mass * vel3[3 * i + 2];
    totalm += mass;
  }
  cmvx = cmvx / totalm;
  cmvy = cmvy / totalm;
  cmvz = cmvz / totalm;
  long s = 0;
  double prev = INFINITY;
  while ((fabs(cmvx) > 1.0e-15) || (fabs(cmvy) > 1.0e-15) || (fabs(cmvz) > 1.0e-15)) {
    double big = fmax(fabs(cmvx), fmax(fabs(cmvy), fabs(cmvz)));
    /* the first shift leaves the pairs' residue; from the second on each
       shift scales the remainder by minus (second atoms' mass) / totalm */
    if (++s > max_shifts || (s > 2 && !(big < prev))) {
      if (shifts) *shifts = s;
      return -1;
    }
    prev = big;
    for (int i = 0; i < n; i++) {
      vel3[3 * i] = vel3[3 * i] - cmvx;
      vel3[3 * i + 1] = vel3[3 * i + 1] - cmvy;
      vel3[3 * i + 2] = vel3[3 * i + 2] - cmvz;
    }
    cmvx = 0.0;
    cmvy = 0.0;
    cmvz = 0.0;
    for (int i = 0; i < n; i++) {
      double mass = mass_of[(int)pos4[4 * i + 3]];
      cmvx = cmvx + vel3[3 * i] * mass;
      cmvy = cmvy + vel3[3 * i + 1] * mass;
      cmvz = cmvz + vel3[3 * i + 2] * mass;
    }
    cmvx = cmvx / totalm;
    cmvy = cmvy / totalm;
    cmvz = cmvz / totalm;
  }
  for (int i = 0; i < n; i++) {
    double mass = mass_of[(int)pos4[4 * i + 3]];
    t += mass * (vel3[3 * i] * vel3[3 * i] + vel3[3 * i + 1] * vel3[3 * i + 1] +
                 vel3[3 * i + 2] * vel3[3 * i + 2]);
  }
  t = t / (3.0 * (double)n);
  double scalev = sqrt(temp / t);
  for (int i = 0; i < n; i++) {
    vel3[3 * i] = vel3[3 * i] * scalev;
    vel3[3 * i + 1] = vel3[3 * i + 1] * scalev;
    vel3[3 * i + 2] = vel3[3 * i + 2] * scalev;
  }
  if (shifts) *shifts = s;
  return k;
}
