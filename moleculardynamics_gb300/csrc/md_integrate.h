// Launch interface of the integrator and reduction kernels (md_integrate.cu).
#pragma once
#include "md_internal.h"

namespace mdgb {

// Gear coefficients of cpu/common/Device.cpp:19-22 and :49-56
struct GearCoef {
  double c1, c2, c3, c4, cr, cv, cb, cc;
};
GearCoef gear_coef(double dt);

struct GearArgs {
  md_double4* pos;
  double* vel;
  double* acc;
  double* b;
  double* c;
  const double* f3;
  int n;
  GearCoef k;
  Species sp;
  float4* posf;            // FP32 copy written after the update (may be NULL)
  const float4* pos_build; // skin reference positions (may be NULL)
  float trip2;             // squared skin displacement
  int* trip;               // trip flag set when an atom exceeds the skin
  int* status;
  int exact;               // 1: the reference's roundings; 0: FMA and 1/m
  double inv_mass[3];
  // correct only
  double npos;
  float energy_loss;
  int walls;
  int* wall_flag;
};

void launch_predict(const GearArgs& a, cudaStream_t st);
void launch_correct(const GearArgs& a, cudaStream_t st);
// correct for this step and predict for the next in one pass (no walls)
void launch_correct_predict(const GearArgs& a, cudaStream_t st);
void launch_accel(const md_double4* pos, double* acc, const double* f3, int n, Species sp,
                  cudaStream_t st);
void launch_posf(const md_double4* pos, float4* posf, int n, cudaStream_t st);
// max |v| and max |coordinate| (cpu/cpumd/Host.cpp:245-271) into umax[0..1]
// as the bit patterns of non-negative doubles; sets ST_NONFINITE.
void launch_ready(const md_double4* pos, const double* vel, int n, unsigned long long* umax,
                  int* status, cudaStream_t st);
// PerformCalculations (common/DebugCalculations.cpp:46-124) into out[0..7]:
// com x,y,z, kinetic, momentum x,y,z, temperature.  part: >= 8 * 1024 doubles.
// chooseVelocities (cpu/equi/Host.cpp:416-572) on the device state (orig:
// caller's numbering of the stored atoms, NULL when stored in it); temp in
// the reference's energy units (kelvin x 8.314e-7); part as for
// launch_thermo.  Returns 0, a CUDA error code, or -1 when a momentum-removal
// shift does not shrink the centre-of-mass velocity (the reference loops on).
int equi_velocities(const md_double4* pos, double* vel, const int* orig, int n, int n_mb,
                    Species sp, double temp, unsigned long long seed, double* part,
                    int* iterations, cudaStream_t st);
void launch_thermo(const md_double4* pos, const double* vel, int n, Species sp, double* part,
                   double* out, cudaStream_t st);
// Deterministic sum of nv-vectors over nblocks partials: out[k] = sum_b part[nv*b + k].
void launch_sum_partials(const double* part, int nblocks, int nv, double* out,
                         cudaStream_t st);
// Per-replica records (16 doubles each, md_thermo layout): thermo of atoms
// [ranges[2k], ranges[2k] + ranges[2k+1]) and LJ energies e3[3k..3k+2]
// (E, E_shifted, W).
void launch_rep_records(const md_double4* pos, const double* vel, const int* ranges, int nrep,
                        Species sp, const double* e3, double time, double step, double* rec,
                        cudaStream_t st);
// calculatePotentional (common/DebugCalculations.cpp:129-270) into out[0..1].
// part: >= 2 * n doubles.
void launch_ref_potential(const md_double4* pos, int n, Species sp, double* part, double* out,
                          cudaStream_t st);
// PerformCalculations and calculatePotentional in the reference's summation
// order (one device thread adds the terms in the reference's sequence), for
// records bit-identical to the reference's: thermo into out8 (layout of
// launch_thermo), the energies into out[0..1].  inv: caller index -> stored
// position (NULL: stored in the caller's order).  buf holds 2 * buf_terms
// doubles; the pair terms go through it in chunks of rows.  Returns the
// number of kernels launched.
void launch_thermo_seq(const md_double4* pos, const double* vel, const int* inv, int n,
                       Species sp, double* out8, cudaStream_t st);
int launch_ref_potential_seq(const md_double4* pos, const int* inv, int n, Species sp,
                             double* buf, long long buf_terms, double* out, cudaStream_t st);
// Assembles an md_thermo record (as 16 doubles) from device scalars:
// th8 from launch_thermo, e_lj3 = (E, E_shifted, W), e_mb3 = (E, W1, W2).
void launch_record(const double* th8, const double* e_lj3, const double* e_mb3,
                   const double* ref2, int use_ref, double time, double step,
                   double* rec16, cudaStream_t st);

}  // namespace mdgb
