/*
 * mdoracle: CPU restatement of the reference MD step (test infrastructure).
 *
 * This is the oracle for the GPU engine: only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline arm may load it, and only as the checker or the
 * timed CPU baseline, never as the product.  It restates, function by
 * function, the FP64 CPU path of vakuras/moleculardynamics (real = double, as
 * cpumd is built) and is pinned bit-for-bit against that reference compiled
 * in place (oracle/build_ref.sh) by tests/test_oracle_pinned.py.
 *
 * Extensions that the reference lacks (each off by default, so that the
 * default behaviour is the reference's):
 *   - periodic cubic box: wrap at list builds, cell wrap in the 27-cell
 *     stencil, periodic image code per list entry;
 *   - species table with the NG slot set to argon;
 *   - potential energy and virial over the same pairs the forces use.
 */
#ifndef MDORACLE_H
#define MDORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Per-species LJ parameters and masses of the NG slot table
 * (common/Constants.h:36-43,55-57).  Values are float literals, promoted to
 * double where used, exactly as the reference does. */
typedef struct {
  float sigNG, sigNGN, sigNGO;
  float epsNG, epsNGN, epsNGO;
  float mN, mO, mNG;
} orc_species;

enum { ORC_SPECIES_NEON = 0, ORC_SPECIES_ARGON = 1 };
void orc_species_get(int which, orc_species* out);

/* Neighbour list in the reference layout (common/NeighborList.cpp:14-156):
 * rows[i*nlistsize + k], -1 padded; code[i*nlistsize + k] is the periodic
 * image of the entry, (ix+1)*9 + (iy+1)*3 + (iz+1) with i* in {-1,0,1}
 * (13 = no shift; always 13 without a periodic box).  cell[3*i] is the
 * build-time cell of atom i. */
typedef struct {
  int n, nlistsize, nlargest, cells, maxcell, periodic;
  double box;   /* reference: boxSizeList; periodic: L */
  int* rows;
  signed char* code;
  int* cell;
} orc_list;

void orc_list_settings(float rs, float rcut, float* maxnlmove, float* maxnlmovesq,
                       float* rcutsq);
void orc_ready_list(const double* pos4, const double* vel3, int n, double* vmax,
                    double* box);
int orc_next_build(float maxnlmove, double vmax, double dt, int t);
/* periodic != 0: L = box edge, positions are wrapped into [-L/2, L/2) first
 * (pos4 is modified).  Returns NULL on allocation failure or bad box. */
orc_list* orc_build_list(double* pos4, int n, float rs, double box, int periodic);
void orc_free_list(orc_list* l);

void orc_predict(double* r4, double* v3, double* a3, double* b3, double* c3, double dt,
                 int nop);
void orc_correct(double* r4, double* v3, const double* f3, double* a3, double* b3,
                 double* c3, double dt, int nop, double npos, int* flag, float energy_loss,
                 int walls, const orc_species* sp);
void orc_accelerations(const double* pos4, double* a3, const double* f3, int n,
                       const orc_species* sp);

/* LJ forces over list rows (cpu/common/LennardJones.h:35-93); overwrites F.
 * With energy != NULL also returns [E, E_shifted, W] over the same pairs
 * (per ordered pair 2 eps (sr^12 - sr^6), and 1/2 r_ij . f_ij). */
void orc_lj_forces(const double* pos4, double* f3, int n, const orc_list* l,
                   double rcutsq, const orc_species* sp, double* energy);
/* Bond-order forces (cpu/common/BondOrderFuncs.h:283-397).  xi scratch is
 * per (i, list slot) instead of N x N.  missing (optional) counts pass-2
 * reads of a xi that pass 1 did not write (undefined in the reference).
 * energy (optional): [E_mb, W_mb] with E_mb = sum over pass-1 pairs of
 * 1/2 (Vr - b Va + Vdw) and W_mb = sum_i r_i . F_i(mb). */
void orc_mb_forces(const double* pos4, double* f3, int mbp, const orc_list* l,
                   double rcutsq, int ljexist, long long* missing, double* energy);

/* common/DebugCalculations.cpp:46 PerformCalculations.
 * out: com x,y,z, kinetic energy, momentum x,y,z, temperature. */
void orc_perform_calculations(const double* pos4, const double* vel3, int n, double* out,
                              const orc_species* sp);
/* common/DebugCalculations.cpp:129 calculatePotentional (all pairs). */
void orc_calculate_potential(const double* pos4, int n, double* vib_lj, double* vib_mb,
                             const orc_species* sp);

typedef struct {
  int n_lj, n_mb, timesteps, use_lj, use_mb, output_timesteps;
  float dt, lj_rs, lj_rcut, mb_rs, mb_rcut, energy_loss, vxcm;
  int periodic;   /* 0: reference walls; 1: periodic cubic box of edge box */
  double box;
  int species;    /* ORC_SPECIES_* */
  int threads;    /* OpenMP threads, 0 = runtime default */
} orc_run_params;

/* One vxcm pass of cpu/cpumd/Host.cpp:hostMain (lines 31-195) on caller
 * arrays, without file I/O.  thermo (optional) gets 12 numbers per record
 * (PerformCalculations' 8, then E_lj, E_lj_shifted, E_mb, W) at t=0 and every
 * output step; returns the number of records.  stats (optional): list
 * builds, wall hits, missing xi reads.  elapsed_ms: wall time of the loop. */
int orc_run(const orc_run_params* p, double* pos4, double* vel3, double* acc3, double* b3,
            double* c3, double* f3, double* thermo, long long* stats, double* elapsed_ms);

int orc_max_threads(void);

/* cpu/equi/Statistics.cpp:115-140 inverf, with the file's own erf/erfc */
double orc_inverf(double z);
/* cpu/equi/Host.cpp:416-572 chooseVelocities with the uniforms given (three
 * per draw); returns the uniforms used, or -1 where the momentum removal does
 * not converge */
long orc_choose_velocities(const double* pos4, double* vel3, int n, int n_mb, double temp,
                           int species, const double* u, long nu, long max_shifts,
                           long* shifts);

#ifdef __cplusplus
}
#endif
#endif
