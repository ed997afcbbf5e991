// Test harness over the reference's equi velocity generator
// (cpu/equi/Host.cpp:416-572 chooseVelocities, cpu/equi/Statistics.cpp:115-140
// inverf), compiled in place by oracle/build_ref.sh into
// oracle/_ref/libmdref_equi_*.so.  Test infrastructure only.
//
// The reference draws from rand() seeded with the clock (cpu/equi/Host.cpp:83);
// the build maps rand() to mdref_replay_rand below, which hands out a stream
// of draws given by the test, so that a run is repeatable and the C
// restatement in oracle/mdoracle.c can be fed the same numbers.
#include "global.h"

void chooseVelocities(real4* posArray, real3* velocityArray, real temp, configuration* config);
double inverf(const double z);

namespace {
const int* g_draws = nullptr;
long g_ndraws = 0, g_next = 0;
}  // namespace

extern "C" {

// the rand() of the compiled equi; 0 once the given stream is used up
int mdref_replay_rand(void) { return g_next < g_ndraws ? g_draws[g_next++] : 0; }

// chooseVelocities on n_lj + n_mb atoms at temp (the reference's units:
// kelvin x 8.314e-7, cpu/equi/Host.cpp:85-86) with the draws given; returns
// how many draws it took.
long ref_equi_choose_velocities(double* pos4, double* vel3, int n_lj, int n_mb, double temp,
                                const int* draws, long ndraws) {
  configuration cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.LennardJonesParticles = n_lj;
  cfg.ManyBodyParticles = n_mb;
  g_draws = draws;
  g_ndraws = ndraws;
  g_next = 0;
  chooseVelocities((real4*)pos4, (real3*)vel3, temp, &cfg);
  return g_next;
}

double ref_equi_inverf(double z) { return inverf(z); }
}
