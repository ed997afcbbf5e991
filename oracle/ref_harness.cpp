// Test harness over the compiled reference engine of vakuras/moleculardynamics.
//
// Test infrastructure only: oracle/build_ref.sh links this file with the
// reference's own object files (built in place, unmodified) into
// oracle/_ref/libmdref_*.so.  The tests load that library to pin the C
// restatement in oracle/mdoracle.c and to generate the golden fixtures in
// tests/golden/.  Every function below forwards to the reference function it
// names; the only logic of its own is ref_run, which replays the body of
// cpu/cpumd/Host.cpp:hostMain (lines 31-195) without file I/O and without the
// O(N^2)/O(N^3) performOutput calls, so that a trajectory can be compared.
#include "host.h"
#include <time.h>

extern "C" {

int ref_real_size(void) { return (int)sizeof(real); }

// cpu/cpumd/Host.cpp:57-61 (LJ) and :66-70 (many-body).
void ref_list_settings(float rs, float rcut, float* maxnlmove, float* maxnlmovesq,
                       float* rcutsq) {
  listSettings s;
  s.maxnlmove = (rs - rcut) * 0.5f;
  s.maxnlmovesq = pow(s.maxnlmove, 2);
  s.rcutsq = pow(rcut, 2);
  *maxnlmove = s.maxnlmove;
  *maxnlmovesq = s.maxnlmovesq;
  *rcutsq = s.rcutsq;
}

// common/NeighborList.cpp:14 buildNeighborList.  Returns the reference's own
// new[]'d list; free it with ref_free_list.
int* ref_build_neighbor_list(const double* pos4, int n, float rs, float rcut,
                             double box, int buckets, int* nlistsize, int* nlargest) {
  listSettings s;
  memset(&s, 0, sizeof(s));
  s.rs = rs;
  s.rcut = rcut;
  int* list = buildNeighborList((real4*)pos4, &s, box, buckets, n);
  *nlistsize = s.nlistsize;
  *nlargest = s.nlargestsize;
  return list;
}

void ref_free_list(int* list) { delete[] list; }

// common/NeighborList.cpp:161 computeBucket on a fresh table, for hash tests.
int ref_compute_bucket_insert(int cx, int cy, int cz, int* table3, int buckets) {
  return computeBucket(cx, cy, cz, (int3*)table3, buckets, false);
}

// cpu/cpumd/Host.cpp:245 readyList.
void ref_ready_list(const double* pos4, const double* vel3, int n, double* vmax,
                    double* box) {
  real hv, bs;
  readyList((real4*)pos4, (real3*)vel3, n, hv, bs);
  *vmax = hv;
  *box = bs;
}

// cpu/cpumd/Host.cpp:276 buildList (list + next build time step).
int* ref_build_list(const double* pos4, float rs, float rcut, double box, int buckets,
                    double vmax, int n, int t, double dt, int* next_build,
                    int* nlistsize, int* nlargest) {
  listSettings s;
  memset(&s, 0, sizeof(s));
  s.maxnlmove = (rs - rcut) * 0.5f;
  s.maxnlmovesq = pow(s.maxnlmove, 2);
  s.rcutsq = pow(rcut, 2);
  s.rcut = rcut;
  s.rs = rs;
  int* list = NULL;
  int nb = 0;
  buildList((real4*)pos4, &s, box, buckets, vmax, n, nb, t, &list, dt);
  *next_build = nb;
  *nlistsize = s.nlistsize;
  *nlargest = s.nlargestsize;
  return list;
}

void ref_predict(double* r4, double* v3, double* a3, double* b3, double* c3, double dt,
                 int nop) {
  predict((real4*)r4, (real3*)v3, (real3*)a3, (real3*)b3, (real3*)c3, dt, nop);
}

void ref_correct(double* r4, double* v3, const double* f3, double* a3, double* b3,
                 double* c3, double dt, int nop, double npos, int* flag,
                 float energy_loss) {
  bool fl = false;
  correct((real4*)r4, (real3*)v3, (real3*)f3, (real3*)a3, (real3*)b3, (real3*)c3, dt, nop,
          npos, fl, energy_loss);
  *flag = fl ? 1 : 0;
}

void ref_lj_forces(const double* pos4, double* f3, int n, int nlargest, int nlistsize,
                   const int* list, double rcutsq) {
  lennardJonesForces((real4*)pos4, (real3*)f3, n, nlargest, nlistsize, (int*)list, rcutsq);
}

void ref_mb_forces(const double* pos4, double* f3, int mbp, int nlargest, int nlistsize,
                   const int* list, double rcutsq, int ljexist) {
  manyBodyForces((real4*)pos4, (real3*)f3, mbp, nlargest, nlistsize, (int*)list, rcutsq,
                 ljexist != 0);
}

void ref_accelerations(const double* pos4, double* a3, const double* f3, int n) {
  calculateAccelerations((real4*)pos4, (real3*)a3, (real3*)f3, n);
}

// out: com x,y,z, kinetic energy, momentum x,y,z, temperature
void ref_perform_calculations(const double* pos4, const double* vel3, int n, double* out) {
  PerformCalculations((real4*)pos4, (real3*)vel3, n, out[0], out[1], out[2], out[3], out[4],
                      out[5], out[6], out[7]);
}

void ref_calculate_potential(const double* pos4, int n, double* vib_lj, double* vib_mb) {
  calculatePotentional((real4*)pos4, vib_lj, vib_mb, n);
}

struct ref_run_params {
  int n_lj, n_mb, timesteps, use_lj, use_mb, output_timesteps;
  float dt, lj_rs, lj_rcut, mb_rs, mb_rcut, energy_loss, vxcm;
};

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

// Replays cpu/cpumd/Host.cpp:hostMain for one vxcm value (lines 31-195) on
// caller arrays.  thermo (optional) receives PerformCalculations' 8 numbers at
// t=0 and at every output step; n_builds counts list builds; elapsed_ms is the
// wall time of the step loop (the reference's own timer spans 130-198).
int ref_run(const ref_run_params* p, double* pos4, double* vel3, double* acc3, double* b3,
            double* c3, double* f3, double* thermo, int* n_builds, double* elapsed_ms) {
  int n = p->n_lj + p->n_mb;
  real4* pos = (real4*)pos4;
  real3* vel = (real3*)vel3;
  real3* a = (real3*)acc3;
  real3* b = (real3*)b3;
  real3* c = (real3*)c3;
  real3* f = (real3*)f3;
  real boxSize = pow(n, 1.0 / 3.0) * 52.8;
  int buckets = n * 3;
  listSettings lj, mb;
  memset(&lj, 0, sizeof(lj));
  memset(&mb, 0, sizeof(mb));
  if (p->use_lj) {
    lj.maxnlmove = (p->lj_rs - p->lj_rcut) * 0.5f;
    lj.maxnlmovesq = pow(lj.maxnlmove, 2);
    lj.rcutsq = pow(p->lj_rcut, 2);
    lj.rcut = p->lj_rcut;
    lj.rs = p->lj_rs;
  }
  if (p->use_mb) {
    mb.maxnlmove = (p->mb_rs - p->mb_rcut) * 0.5f;
    mb.maxnlmovesq = pow(mb.maxnlmove, 2);
    mb.rcutsq = pow(p->mb_rcut, 2);
    mb.rcut = p->mb_rcut;
    mb.rs = p->mb_rs;
  }
  float energyLoss = sqrt(p->energy_loss);
  int* ljList = NULL;
  int* mbList = NULL;
  int timesteps = 0, ljNextBuild = 0, mbNextBuild = 0, builds = 0, nth = 0;
  real highestVelocity, boxSizeList;
  memset(a, 0, sizeof(real3) * n);
  memset(b, 0, sizeof(real3) * n);
  memset(c, 0, sizeof(real3) * n);
  for (int id = 0; id < n; id++) {
    if (fabs(pos[id].x) > (boxSize / 2)) pos[id].x = (boxSize / 2) * (pos[id].x / fabs(pos[id].x));
    if (fabs(pos[id].y) > (boxSize / 2)) pos[id].y = (boxSize / 2) * (pos[id].y / fabs(pos[id].y));
    if (fabs(pos[id].z) > (boxSize / 2)) pos[id].z = (boxSize / 2) * (pos[id].z / fabs(pos[id].z));
    vel[id].x += p->vxcm;
  }
  readyList(pos, vel, n, highestVelocity, boxSizeList);
  if (p->use_lj) { buildList(pos, &lj, boxSizeList, buckets, highestVelocity, n, ljNextBuild, 0, &ljList, p->dt); builds++; }
  if (p->use_mb) { buildList(pos, &mb, boxSizeList, buckets, highestVelocity, p->n_mb, mbNextBuild, 0, &mbList, p->dt); builds++; }
  if (thermo) ref_perform_calculations(pos4, vel3, n, thermo + 8 * nth++);
  double t0 = now_ms();
  if (p->use_lj) lennardJonesForces(pos, f, n, lj.nlargestsize, lj.nlistsize, ljList, lj.rcutsq);
  if (p->use_mb) manyBodyForces(pos, f, p->n_mb, mb.nlargestsize, mb.nlistsize, mbList, mb.rcutsq, p->use_lj != 0);
  calculateAccelerations(pos, a, f, n);
  int printout = p->output_timesteps;
  while (timesteps < p->timesteps) {
    if (ljNextBuild == timesteps || mbNextBuild == timesteps) {
      readyList(pos, vel, n, highestVelocity, boxSizeList);
      if (p->use_lj && ljNextBuild == timesteps) { buildList(pos, &lj, boxSizeList, buckets, highestVelocity, n, ljNextBuild, timesteps, &ljList, p->dt); builds++; }
      if (p->use_mb && mbNextBuild == timesteps) { buildList(pos, &mb, boxSizeList, buckets, highestVelocity, p->n_mb, mbNextBuild, timesteps, &mbList, p->dt); builds++; }
    }
    predict(pos, vel, a, b, c, p->dt, n);
    if (p->use_lj) lennardJonesForces(pos, f, n, lj.nlargestsize, lj.nlistsize, ljList, lj.rcutsq);
    if (p->use_mb) manyBodyForces(pos, f, p->n_mb, mb.nlargestsize, mb.nlistsize, mbList, mb.rcutsq, p->use_lj != 0);
    bool flag = false;
    correct(pos, vel, f, a, b, c, p->dt, n, boxSize, flag, energyLoss);
    if (flag) {
      if (p->use_lj) lennardJonesForces(pos, f, n, lj.nlargestsize, lj.nlistsize, ljList, lj.rcutsq);
      if (p->use_mb) manyBodyForces(pos, f, p->n_mb, mb.nlargestsize, mb.nlistsize, mbList, mb.rcutsq, p->use_lj != 0);
      calculateAccelerations(pos, a, f, n);
    }
    if (printout == timesteps) {
      if (thermo) ref_perform_calculations(pos4, vel3, n, thermo + 8 * nth++);
      printout += p->output_timesteps;
    }
    timesteps++;
  }
  *elapsed_ms = now_ms() - t0;
  *n_builds = builds;
  if (ljList) delete[] ljList;
  if (mbList) delete[] mbList;
  return nth;
}

// common/Loader.cpp:34 readConfiguration.  Flattens the struct for ctypes:
// ints  = LJ particles, MB particles, Timesteps, CudaBlocks, OutputTimesteps,
//         AnimationTimesteps, UseCuda, UseLJ, UseMB, LJBPP, MBBPP, Debug, Fallback
// floats= DT, Temperature, LJRS, LJRCUT, MBRS, MBRCUT, VXCMFROM, VXCMTO,
//         VXCMSTEP, EnergyLoss
// strs  = Input, Output, Filename, AnimationData, each in a 256-byte slot.
void ref_read_configuration(const char* path, int* ints, float* floats, char* strs) {
  configuration cfg;
  readConfiguration(string(path), &cfg);
  int iv[13] = {cfg.LennardJonesParticles, cfg.ManyBodyParticles, cfg.Timesteps,
                cfg.CudaBlocks, cfg.OutputTimesteps, cfg.animts, cfg.UseCuda,
                cfg.useLennardJones, cfg.useManyBody, cfg.lennardJonesBPP,
                cfg.manyBodyBPP, cfg.Debug, cfg.Fallback};
  float fv[10] = {cfg.DT, cfg.Temperature, cfg.LennardJonesRS, cfg.LennardJonesRCUT,
                  cfg.ManyBodyRS, cfg.ManyBodyRCUT, cfg.vxcmFrom, cfg.vxcmTo,
                  cfg.vxcmStep, cfg.energyLoss};
  memcpy(ints, iv, sizeof(iv));
  memcpy(floats, fv, sizeof(fv));
  const string* sv[4] = {&cfg.Input, &cfg.Output, &cfg.Filename, &cfg.AnimFile};
  for (int k = 0; k < 4; k++) {
    strncpy(strs + 256 * k, sv[k]->c_str(), 255);
    strs[256 * k + 255] = 0;
  }
}

// common/Results.cpp:120 writeResults with common/Results.cpp:88 tailResults.
// records: nrec x 11 doubles in the order of struct results (Results.h:15-28).
void ref_write_results(const char* filename, int n_lj, int n_mb, int timesteps, float dt,
                       int use_lj, float lj_rs, float lj_rcut, int use_mb, float mb_rs,
                       float mb_rcut, float vxcm, float elapsed, const double* records,
                       int nrec, const double* pos4) {
  configuration cfg;
  cfg.LennardJonesParticles = n_lj;
  cfg.ManyBodyParticles = n_mb;
  cfg.Timesteps = timesteps;
  cfg.DT = dt;
  cfg.useLennardJones = use_lj != 0;
  cfg.LennardJonesRS = lj_rs;
  cfg.LennardJonesRCUT = lj_rcut;
  cfg.useManyBody = use_mb != 0;
  cfg.ManyBodyRS = mb_rs;
  cfg.ManyBodyRCUT = mb_rcut;
  cfg.Filename = filename;
  vector<results> rv(nrec);
  memcpy(&rv[0], records, sizeof(results) * nrec);
  writeResults(rv, &cfg, elapsed, tailResults((real4*)pos4, n_mb), vxcm);
}

// common/Loader.cpp:88 writeOutput and :125 readInput.
void ref_write_output(const char* path, int n, const double* pos4, const double* vel3) {
  configuration cfg;
  cfg.LennardJonesParticles = n;
  cfg.ManyBodyParticles = 0;
  cfg.Output = path;
  writeOutput(&cfg, (real*)pos4, (real*)vel3);
}

void ref_read_input(const char* path, int n, double* pos4, double* vel3) {
  configuration cfg;
  cfg.LennardJonesParticles = n;
  cfg.ManyBodyParticles = 0;
  cfg.Input = path;
  readInput(&cfg, (real*)pos4, (real*)vel3);
}

}  // extern "C"
