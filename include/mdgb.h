/*
 * mdgb.h: C ABI of the GB300 (sm_103a) MD step engine (libmdgb.so).
 *
 * Drop-in for the step loop of vakuras/moleculardynamics' cpumd
 * (cpu/cpumd/Host.cpp:114-195): neighbour-list build, Lennard-Jones and
 * bond-order forces, Gear predictor-corrector, energy/virial reduction.
 *
 * Two layers, both plain C (pointers and sizes only):
 *
 *  1. Engine API (md_*): a context that owns the state on the device and runs
 *     whole steps there.  Host arrays use the reference's layouts: positions
 *     real4 = (x, y, z, type), vectors real3, real = double
 *     (common/Global.h:58-72).  Every call returns an md_status; nothing
 *     exits the process (the reference exits on any error, Global.h:116-117).
 *     One context per host thread; a context is not re-entrant.
 *
 *  2. Reference-signature API (mdgb_*): the functions of cpu/common/Device.h,
 *     common/NeighborList.h and common/DebugCalculations.h with the same
 *     arguments and meaning, operating on host arrays (each call copies in,
 *     computes on the GPU, copies out).  A C++ file that forwards the
 *     reference names to these (refshim/cpumd_device_gb300.cpp in this
 *     package) is all cpumd needs.  They return void like the reference;
 *     mdgb_last_status() reports failures.
 *
 * Units are the reference's: angstrom, femtosecond, g/mol, energy 1e7 J/mol.
 */
#ifndef MDGB_H
#define MDGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum md_status {
  MD_OK = 0,
  MD_BAD_CONFIG = 1,     /* invalid configuration value */
  MD_LIST_OVERFLOW = 2,  /* caller buffer too small for the neighbour list */
  MD_NONFINITE = 3,      /* NaN/inf in positions, velocities or forces */
  MD_TIMEOUT = 4,        /* a bounded device wait gave up */
  MD_CUDA_ERROR = 5,     /* CUDA runtime error (see md_last_error) */
  MD_BAD_ARGUMENT = 6,   /* NULL pointer, bad index or size */
  MD_NO_DEVICE = 7,      /* no usable CUDA device */
  MD_OUT_OF_MEMORY = 8,  /* device allocation failed */
  MD_CELL_OVERFLOW = 9   /* cell grid out of range (atoms far outside the box) */
} md_status;

enum { MD_PREC_FP64 = 0, MD_PREC_MIXED = 1 };
enum { MD_SPECIES_NEON = 0, MD_SPECIES_ARGON = 1 };

/* Configuration.  The first block is the subset of the reference's
 * `configuration` (common/Global.h:75-104, keys in common/Loader.h:25-51)
 * that the step uses; the second block are extensions whose zero value is
 * the reference's behaviour. */
typedef struct md_config {
  int n_lj;                /* "Lennard Jones Particles" */
  int n_mb;                /* "Many Body Particles": atoms [0, n_mb) are many-body */
  float dt;                /* "DT" */
  int timesteps;           /* "Timesteps" */
  float lj_rs, lj_rcut;    /* "LennardJonesRS", "LennardJonesRCUT" */
  float mb_rs, mb_rcut;    /* "ManyBodyRS", "ManyBodyRCUT" */
  int use_lj, use_mb;      /* "UseLennardJones", "UseManyBody" */
  int output_timesteps;    /* "OutputTimesteps" (<= 0: no records) */
  float energy_loss;       /* "EnergyLoss"; its square root is used (Host.cpp:73) */
  /* extensions */
  int periodic;            /* 1: periodic cubic box of edge `box`, no walls */
  double box;
  int precision;           /* MD_PREC_FP64 (plain) or MD_PREC_MIXED (FP32 pairs) */
  int species;             /* MD_SPECIES_NEON (reference table) or _ARGON (NG = argon) */
  int device;              /* CUDA device ordinal */
  int reference_energy;    /* 1: records use the reference's all-pairs energy
                              (DebugCalculations.cpp:129-270, O(N^2)/O(N^3));
                              2: the same, and every record quantity summed in the
                              reference's order by one device thread (records
                              bit-identical to the reference's for LJ systems; for
                              small systems) */
  int lj_kernel;           /* MD_LJ_AUTO, MD_LJ_ROWS or MD_LJ_CLUSTER (precision form) */
  int cluster_cells;       /* cells per segment of the cluster kernel (0: default) */
  int cluster_threads;     /* threads per segment block (0: default; multiple of 32, <= 224) */
  int cluster_row_loads;   /* rows of the cluster kernel: 0 default / autotuned, 1 TMA tiles of
                              the block in shared memory (two in flight), 2 per-lane register
                              prefetch, 3 TMA tiles of each warp, 4 as 1 with three in flight */
  int cluster_stage_cap;   /* staged atoms per segment of the cluster kernel (0: default /
                              autotuned; otherwise 64 .. 11264) */
} md_config;

/* LJ kernel of the precision form.  ROWS: compact rows of packed atom
 * indices streamed by TMA, positions gathered from L2.  CLUSTER (periodic,
 * LJ only): atoms sorted by cell, each block stages the positions of a
 * segment's neighbour cells in shared memory and rows hold 16-bit offsets
 * into it; the state is kept in that order on the device and mapped back to
 * the caller's numbering at every download.  AUTO picks CLUSTER where it
 * applies. */
enum { MD_LJ_AUTO = 0, MD_LJ_ROWS = 1, MD_LJ_CLUSTER = 2 };

/* One output record.  The first 11 doubles are the reference's `results`
 * (common/Results.h:15-28) in the same order; eu is the potential energy
 * (list energy, or the all-pairs one with reference_energy). */
typedef struct md_thermo {
  double time, temperature, e, ek, eu;
  double com_x, com_y, com_z;
  double momentum_x, momentum_y, momentum_z;
  double e_lj;             /* LJ energy over the force's pairs (within rcut) */
  double e_lj_shifted;     /* same, each pair shifted by its value at rcut */
  double e_mb;             /* bond-order energy over the force's pairs */
  double virial;           /* W = 1/2 sum r_ij.f_ij (LJ) + sum r_i.F_i (bond order) */
  double step;
} md_thermo;

typedef struct md_stats {
  long long steps;
  long long list_builds;
  long long list_trips;    /* steps that walked full rows (skin exceeded) */
  long long wall_hits;     /* steps with a wall reflection (Device.cpp:86-118) */
  long long missing_xi;    /* pass-2 reads of an xi pass 1 did not make */
  long long launches;      /* kernels launched by this context */
  int lj_max_row;          /* longest compact LJ row at the last build */
  int lj_nlargest;         /* longest full LJ candidate row (nlargestsize) */
  int mb_nlargest;
  int lj_cells, mb_cells;
  long long lj_list_entries; /* entries of the compact LJ list at the last build */
  int lj_tma;              /* 1: the LJ list is streamed by TMA (precision form) */
  int lj_cluster;          /* 1: the cluster kernel computes LJ (precision form) */
  int cluster_segments;    /* segment blocks of the cluster kernel */
  int cluster_max_staged;  /* largest staged neighbourhood (atoms) */
} md_stats;

typedef struct md_ctx md_ctx;

/* ---- engine API ---- */
md_status md_create(const md_config* cfg, md_ctx** out);
void md_destroy(md_ctx* ctx);
const char* md_status_string(md_status s);
const char* md_last_error(const md_ctx* ctx);

/* Positions (n x real4) and velocities (n x real3), n = n_lj + n_mb.
 * Replaces readInput into posArray/velocityArray (common/Loader.cpp:125). */
md_status md_upload(md_ctx* ctx, const double* pos4, const double* vel3);
/* Full Gear state in/out (checkpoint): acc, b, c as n x real3; any may be NULL. */
md_status md_upload_state(md_ctx* ctx, const double* pos4, const double* vel3,
                          const double* acc3, const double* b3, const double* c3);
md_status md_download(md_ctx* ctx, double* pos4, double* vel3);
md_status md_download_state(md_ctx* ctx, double* acc3, double* b3, double* c3,
                            double* force3);

/* Start of one vxcm pass of hostMain (cpu/cpumd/Host.cpp:86-138): zero the
 * Gear derivatives, clamp into the box (or wrap, periodic), add vxcm to vx,
 * build the lists, initial forces and a = F/m, record t = 0. */
md_status md_begin(md_ctx* ctx, float vxcm);
/* nsteps iterations of the step loop (cpu/cpumd/Host.cpp:141-195). */
md_status md_step(md_ctx* ctx, int nsteps);

/* Output records collected at t = 0 and every output step. */
int md_record_count(const md_ctx* ctx);
md_status md_get_records(md_ctx* ctx, md_thermo* out, int max_records);
/* performOutput (common/DebugCalculations.cpp:14-41) on the current state. */
md_status md_thermo_now(md_ctx* ctx, md_thermo* out);
/* calculatePotentional (common/DebugCalculations.cpp:129-270) on the device. */
md_status md_reference_potential(md_ctx* ctx, double* vib_lj, double* vib_mb);
/* Forces at the current positions as Host.cpp:132-135 computes them, plus
 * [E_lj, E_lj_shifted, W_lj, E_mb, W_mb] (energy5 may be NULL). */
md_status md_compute_forces(md_ctx* ctx, double* force3, double* energy5);
/* Neighbour list in the reference layout (NeighborList.cpp:119-177): which =
 * 0 (LJ) or 1 (many-body); rows[i * nlistsize + k], -1 padded; images
 * (optional, same shape, periodic image (ix+1)*9+(iy+1)*3+(iz+1), 13 = none).
 * capacity is the number of ints rows can hold. */
md_status md_neighbor_list(md_ctx* ctx, int which, int* rows, signed char* images,
                           long long capacity, int* nlistsize, int* nlargest);
md_status md_get_stats(const md_ctx* ctx, md_stats* out);
/* Per-kernel device timing with CUDA events on the engine's stream.
 * kernel: 0 = LJ force, 1 = bond order, 2 = predict, 3 = correct, 4 = list build,
 * 5 = whole md_step calls (first launch to last), 6 = cluster force kernel with the
 * Gear correct + predict fused in (precision form, periodic), 7 = the same kernel with
 * the correct only (the steps before a list build, a record or the call's end). */
md_status md_set_timing(md_ctx* ctx, int on);
md_status md_kernel_time(const md_ctx* ctx, int kernel, double* total_ms, long long* launches);
/* Autotuner of the cluster kernel (precision form, periodic): times `evals`
 * launches of the kernel the steps use (the fused force + Gear kernel in the
 * precision form, on a scratch copy of the Gear state) on the current state
 * for each candidate block size, staged-atom cap per segment and row-load
 * scheme, keeps the fastest and rebuilds the list with it.  The caps tried
 * are 1152, 1536 and, per block size and scheme, the largest at which the
 * kernel keeps the blocks per SM that its registers allow.  Forces do not
 * depend on the choice (same pairs, same order).  No-op for the other
 * kernels.  Call after md_begin, best on a thermalised state: on a perfect
 * lattice every row has the same length, which favours other tilings. */
typedef struct md_tune_result {
  int threads;             /* threads per segment block */
  int stage_cap;           /* staged atoms per segment (cap of the column cut) */
  int row_loads;           /* 1 block TMA tiles, 2 register prefetch, 3 warp TMA tiles,
                              4 block TMA tiles three deep */
  int candidates;          /* configurations timed */
  double best_ms;          /* launch time of the choice: the fused force + Gear kernel where
                              steps fuse (precision form), else the force kernel */
} md_tune_result;
md_status md_autotune(md_ctx* ctx, int evals, md_tune_result* out);
/* CUDA graphs for the cluster path (default on): windows of fused steps
 * with nothing else due are replayed as one captured graph. */
md_status md_set_graphs(md_ctx* ctx, int on);
/* Bounded device waits of the LJ kernels: a wait on an mbarrier for a TMA
 * row tile or a staged neighbourhood gives up after `tries` polls, the call
 * returns MD_TIMEOUT, and the kernel leaves once the copies it still has in
 * flight have landed (those last waits keep the default limit, so no copy
 * outlives its block).  Default 1 << 20; tries = 0 gives up at the first
 * wait (for tests of the timeout path).  The surrogate's tensor-core commit
 * waits always use the default.  The state after MD_TIMEOUT is undefined:
 * upload it again before stepping on. */
md_status md_set_wait_limit(md_ctx* ctx, int tries);

/* Arithmetic peaks of a device measured with CUDA events: dependent FMA
 * chains on every SM, FMA = 2 flops (the roofline denominators of the FP64
 * and FP32 kernels).  Takes about 0.1 s. */
md_status md_measure_arith_peaks(int device, double* fp64_gflops, double* fp32_gflops);
md_status md_device_sm_count(int device, int* sms);

/* ---- batched form: many independent periodic replicas in one context ----
 * Replica k has natoms[k] atoms in a cubic periodic box of edge boxes[k];
 * its atoms are the k-th consecutive range of the arrays given to
 * md_upload / md_download (real4 / real3, in replica order).  cfg gives the
 * shared settings (dt, list radii, species); it must select the precision
 * form (MD_PREC_MIXED), LJ only, and output_timesteps <= 0 (records come
 * from md_batch_records).  Every step of all replicas is one launch of the
 * persistent cluster kernel (forces + Gear), replayed from CUDA graphs
 * between list builds; md_step, md_autotune, md_get_stats and the timing
 * calls work on the batch as on any context.  No counterpart in the
 * reference, which runs one system per process (cpu/cpumd/Host.cpp). */
md_status md_batch_create(const md_config* cfg, int nrep, const int* natoms,
                          const double* boxes, md_ctx** out);
int md_batch_size(const md_ctx* ctx);
/* One record per replica of the current state (md_thermo layout; eu = the
 * replica's LJ energy over the force's pairs, e_mb = 0). */
md_status md_batch_records(md_ctx* ctx, md_thermo* out, int max_records);

/* ---- learned surrogate of the bond-order term (no counterpart in the
 * reference) ----
 * Per-atom descriptors: 16 radial and 16 angular Behler symmetry functions
 * (FP32) of the neighbours within `cutoff` (at most the bond-order RCUT).
 * Network: 32-64-64-1 MLP (tanh) giving a per-atom energy; BF16 weights on
 * the tensor cores (tcgen05) with FP32 accumulation; forces from its
 * analytic gradient.  Trained with Adam on per-atom energies of the exact
 * method: E_i = sum_j 1/2 (Vr - b Va + Vdw) over i's bond-order pairs.
 * Attached to a context, it replaces the exact bond-order forces while its
 * force error, measured against the exact kernel every check_every steps
 * (relative RMS over the bond-order atoms), stays within threshold; the
 * exact kernel computes the forces otherwise. */
typedef struct md_surrogate md_surrogate;
typedef struct md_surrogate_stats {
  long long surrogate_steps;   /* steps whose bond-order forces came from the network */
  long long exact_steps;       /* steps that used the exact kernel */
  long long checks;            /* exact-kernel checks of the network */
  long long rejected_checks;   /* checks whose error exceeded the threshold */
  double last_error;           /* relative RMS force error at the last check */
  double max_error;            /* the largest of them since md_surrogate_attach */
  long long declined_steps;    /* steps (checks included) on which some atom's descriptors
                                  lay outside the training data's range: exact forces */
} md_surrogate_stats;
md_status md_surrogate_create(int device, unsigned long long seed, float cutoff,
                              md_surrogate** out);
void md_surrogate_destroy(md_surrogate* s);
int md_surrogate_param_count(void);
/* appends bond-order atoms offset, offset + stride, ... of ctx's current
 * state (descriptors + exact per-atom energies) to the training set, and the
 * whole state (positions, neighbours, exact forces and energies) to the
 * force-matching configurations */
md_status md_surrogate_collect(md_surrogate* s, md_ctx* ctx, int stride, int offset, int* added);
md_status md_surrogate_samples(const md_surrogate* s, int* count);
/* Adam steps on random batches of the training set; *loss = mean squared
 * error of the normalised per-atom energy over the last steps */
md_status md_surrogate_train(md_surrogate* s, int steps, int batch, float lr, double* loss);
/* force matching over the collected configurations (one per Adam step):
 * loss = w_energy * mean((t - t*)^2) + w_force * mean(|F - F*|^2) / var(F*),
 * t the normalised per-atom energy, F the bond-order forces; the losses of
 * the last pass over the configurations come back in loss_energy/loss_force */
md_status md_surrogate_train_forces(md_surrogate* s, int steps, float lr, float w_energy,
                                    float w_force, double* loss_energy, double* loss_force);
/* s = NULL detaches */
md_status md_surrogate_attach(md_ctx* ctx, md_surrogate* s, double threshold, int check_every);
md_status md_surrogate_report(const md_ctx* ctx, md_surrogate_stats* out);
/* network bond-order forces (n_mb x real3) and energy at ctx's state */
md_status md_surrogate_forces(md_surrogate* s, md_ctx* ctx, double* force3, double* energy);
/* descriptors (n_mb x 32): raw, or normalised as the network sees them */
md_status md_surrogate_descriptors(md_surrogate* s, md_ctx* ctx, float* g, int normalised);
/* q[i][f] = sum_j (e_j - e_i) . dG_if/dd_j: the derivative of the raw
 * descriptors of the first n_mb atoms when every atom moves along e3
 * (n_mb x 3); q is n_mb x 32.  The force-matching gradient applies this
 * product to the force residual. */
md_status md_surrogate_desc_directional(md_surrogate* s, md_ctx* ctx, const double* e3,
                                        double* q);
/* FP32 parameters: W1 [64][32], b1 [64], W2 [64][64], b2 [64], w3 [64], b3 */
md_status md_surrogate_params(md_surrogate* s, float* params, int set);
/* input normalisation (x = (g - mean) * istd) and target scaling
 * (E = mu + sigma * t), mu_sigma = {mu, sigma} */
md_status md_surrogate_normalisation(md_surrogate* s, float* mean32, float* istd32,
                                     double* mu_sigma, int set);
/* loss = mean over rows of (net(x) - t)^2 and its gradient (FP32, same
 * layout as the parameters), from the training kernels */
md_status md_surrogate_loss_grad(md_surrogate* s, const float* x, const float* t, int n,
                                 float* grad, double* loss);
/* parameter gradient of sum_i v_i . dt/dx(x_i) (the force-matching term of
 * the training kernels) for normalised inputs x and directions v (n x 32) */
md_status md_surrogate_force_grad(md_surrogate* s, const float* x, const float* v, int n,
                                  float* grad);
/* network output t (n) and dt/dx (n x 32) for normalised inputs x (n x 32) */
md_status md_surrogate_net(md_surrogate* s, const float* x, int n, float* t, float* dtdx);
/* Model kind, before training: 0 (default) the per-atom energy network above
 * (BF16 tcgen05, forces from its gradient); 1 a direct-force head: a
 * 32 -> hidden -> hidden -> 32 FP32 network (tanh; hidden 32, 64 or 128) whose
 * outputs w_i, scaled by the output scale s_out and the descriptor
 * normalisation istd, stand where dE_i/dG_i stands for the energy network:
 * F_j = -sum_i (w_i s_out istd) . dG_i/dr_j.  Nothing makes these forces a
 * gradient, so they can follow the reference's non-conservative bond-order
 * forces; the head has no energy (md_surrogate_forces reports NaN).  It is
 * trained by md_surrogate_train_forces (force matching; w_energy is
 * ignored).  Its hidden weights start from the surrogate's seed, its output
 * layer at zero. */
md_status md_surrogate_set_model(md_surrogate* s, int kind, int hidden);
/* s_out, the forces of one unit of head output: the force RMS of the
 * training data over the force RMS that unit-variance outputs give on the
 * first training configuration, measured at the first training after a
 * normalisation (set = 0 reads it, 0 before then; set = 1 restores a saved
 * value together with md_surrogate_head_params) */
md_status md_surrogate_head_scale(md_surrogate* s, double* scale, int set);
/* The descriptor range the attached surrogate accepts (32 normalised lower
 * and upper bounds).  md_surrogate_train_forces sets it to the range of the
 * stored configurations, widened by a tenth of each span; while it is set, a
 * step on which any atom's descriptors fall outside it takes the exact
 * kernel's forces, and a check on such a step fails.  set = 0 reads it
 * (MD_BAD_ARGUMENT before any training), set = 1 restores a saved one. */
md_status md_surrogate_range(md_surrogate* s, float* lo32, float* hi32, int set);
/* parameters of the direct-force head: W1 [h][32], b1 [h], W2 [h][h], b2 [h],
 * W3 [32][h], b3 [32]; count must be md_surrogate_head_param_count(hidden) */
int md_surrogate_head_param_count(int hidden);
md_status md_surrogate_head_params(md_surrogate* s, float* params, int count, int set);
/* parameter gradient of sum_i v_i . w(x_i) of the head (x, v: n x 32 host
 * arrays), for the comparison with the CPU restatement */
md_status md_surrogate_head_grad(md_surrogate* s, const float* x, const float* v, int n,
                                 float* grad);

/* Tensor-core self-test (no counterpart in the reference): c[128 x ncols] =
 * a[128 x kdim] * b[ncols x kdim]^T on tcgen05 with BF16 operands rounded to
 * nearest from the FP32 inputs and FP32 accumulation; row-major host arrays;
 * ncols in {32, 64, 128}, kdim a multiple of 16 up to 128. */
md_status mdgb_tc_selftest(const float* a, const float* b, float* c, int ncols, int kdim);

/* Self-test of the integer-operation conversions of the fused Gear update:
 * wide[i] = widen(f[i]) (FP32 -> FP64, exact) and narrow[i] = narrow(d[i])
 * (FP64 -> FP32, nearest-even), each beside the conversion instruction's
 * result (wide_ref, narrow_ref), for count values on the device. */
md_status mdgb_conv_selftest(const float* f, const double* d, int count, double* wide,
                             double* wide_ref, float* narrow, float* narrow_ref);

/* Wait for all work of the context; returns the first deferred error. */
md_status md_synchronize(md_ctx* ctx);
/* Page-locked host memory for fast md_upload/md_download (NULL on failure). */
void* md_host_alloc(size_t bytes);
void md_host_free(void* p);

/* ---- reference-signature API ---- */
typedef struct mdgb_list_settings { /* common/NeighborList.h:19-28 listSettings */
  float maxnlmove, maxnlmovesq, rcut, rs, rcutsq;
  int nlistsize, nlargestsize;
} mdgb_list_settings;

/* cpu/common/Device.h:19 predict */
void mdgb_predict(double* r4, double* v3, double* a3, double* b3, double* c3, double dt,
                  int nop);
/* cpu/common/Device.h:20 correct; *flag set to 1 on a wall hit */
void mdgb_correct(double* r4, double* v3, const double* f3, double* a3, double* b3,
                  double* c3, double dt, int nop, double npos, int* flag, float energy_loss);
/* cpu/common/Device.h:21 lennardJonesForces (list in the reference layout) */
void mdgb_lennard_jones_forces(const double* pos4, double* f3, int n, int nlargestsize,
                               int nlistsize, const int* list, double rcutsq);
/* cpu/common/Device.h:22 manyBodyForces */
void mdgb_many_body_forces(const double* pos4, double* f3, int n, int nlargestsize,
                           int nlistsize, const int* list, double rcutsq, int ljexist);
/* cpu/common/Device.h:23 calculateAccelerations */
void mdgb_calculate_accelerations(const double* pos4, double* a3, const double* f3, int n);
/* common/NeighborList.h:30 buildNeighborList; returns a malloc'd list that
 * the caller frees with mdgb_free (the reference returns new int[]) */
int* mdgb_build_neighbor_list(const double* pos4, mdgb_list_settings* s, double box,
                              int buckets, int n);
void mdgb_free(void* p);
/* common/DebugCalculations.h:18 PerformCalculations */
void mdgb_perform_calculations(const double* pos4, const double* vel3, int n, double* com_x,
                               double* com_y, double* com_z, double* kinetic,
                               double* mom_x, double* mom_y, double* mom_z, double* temp);
/* common/DebugCalculations.h:20 calculatePotentional */
void mdgb_calculate_potential(const double* pos4, double* vib_lj, double* vib_mb, int n);
/* Bond-order forces as mdgb_many_body_forces computes them, on DEVICE arrays,
 * without allocating any GPU memory.  No counterpart in the reference: it is
 * for callers that may not allocate device memory themselves, such as a host
 * application that hands out all GPU memory from its own pool and forbids
 * direct cudaMalloc/cudaFree, or a time-critical loop that cannot take the
 * synchronisation an allocation may cause.  Inputs and the output are the
 * caller's device arrays: d_pos4 (n x real4, 32-byte aligned), d_list (rows in
 * the reference layout), d_f3 (n x real3; overwritten when ljexist is 0,
 * accumulated into when it is 1).  d_missing_xi (device int, may be NULL)
 * receives the number of third-body reads of a xi that pass 1 did not make
 * (a list built at other positions; those xi count as 0), as the regular
 * path reports missing_xi.  Scratch lives in one fixed array of about 24 MB
 * inside the library, held on every GPU that loads it until the process
 * exits; sizes above 16384 atoms or 1048576 atom x row-slot pairs
 * (n * nlargestsize) are rejected with MD_BAD_ARGUMENT and a message in err.
 * Each call looks up the array's address on the current device (no
 * allocation); the first call on a device also loads the library's device
 * image there, so make that first call before any stream capture.  All calls
 * share the array: calls that overlap on the GPU race, so serialise them.
 * stream is a cudaStream_t (NULL: the default stream); the work is queued on
 * it and the function returns without waiting.  Returns md_status. */
int mdgb_many_body_forces_static(const double* d_pos4, double* d_f3, int n, int nlargestsize,
                                 int nlistsize, const int* d_list, double rcutsq, int ljexist,
                                 int* d_missing_xi, void* stream, char* err, int err_len);
/* species table of the mdgb_* layer: MD_SPECIES_NEON (default, the reference's) */
void mdgb_set_species(int species);
/* status of the last mdgb_* call on this thread (MD_OK or the failure) */
int mdgb_last_status(void);

/* ---- configuration and results files (common/ConfigParser, Loader, Results) ---- */
/* Reads a reference config file (key=value, '//' comments, keys case-
 * insensitive; the 25 mandatory keys of common/Loader.cpp:49-82) into cfg;
 * strings (Input, Output, Filename, AnimationData) into 4 slots of 512 bytes;
 * extra[0..5] = Temperature, VXCMFROM, VXCMTO, VXCMSTEP, CUDA Blocks, AnimationTimesteps.
 * Optional extension keys: Periodic, Box, Precision, Species, Device. */
md_status md_read_config(const char* path, md_config* cfg, char* strings, double* extra,
                         char* err, int err_len);
/* Writes the .dat/.txt result pair of common/Results.cpp:120-229; the
 * many-body pair list of the .txt (tailResults, common/Results.cpp:88-118)
 * is computed on the host from pos4. */
md_status md_write_results(const char* filename, const md_config* cfg, float vxcm,
                           float elapsed_ms, const md_thermo* records, int nrec,
                           const double* pos4);
/* The same files with the pair list given: pairs[2k], pairs[2k + 1] for
 * k < npairs (from md_tail_pairs). */
md_status md_write_results_pairs(const char* filename, const md_config* cfg, float vxcm,
                                 float elapsed_ms, const md_thermo* records, int nrec,
                                 const int* pairs, int npairs);

/* ---- run outputs on the device (common/Results.cpp) ---- */
/* Animation frames (pushAnim and writeAnimationBinaryData,
 * common/Results.cpp:12-31,51-86).  every >= 0 captures a frame at md_begin
 * and then at steps every, 2 every, ... (every = 0: one more frame at step 0,
 * as cpu/cpumd/Host.cpp:83,126,188-192 behave); every < 0 stops capturing.
 * A frame is the state converted to float on the device and copied to
 * pinned host memory on a copy stream, so capturing does not stop the step
 * loop; frames_hint sizes the first pinned block (more are allocated when a
 * run outgrows it).  md_begin starts a new set of frames. */
md_status md_set_animation(md_ctx* ctx, int every, int frames_hint);
int md_animation_count(const md_ctx* ctx);
/* frame k: n x float4 positions (x, y, z, type) and n x float3 velocities
 * in the caller's numbering (either pointer may be NULL) */
md_status md_get_animation_frame(md_ctx* ctx, int k, float* pos4, float* vel3);
/* writes "<anim_file>(vxcm-<vxcm>).anm": int atoms, int animation steps,
 * int frames, every frame's positions, then every frame's velocities */
md_status md_write_animation(md_ctx* ctx, const char* anim_file, float vxcm);
/* ---- equi: initial velocities (cpu/equi/Host.cpp:416-572) ---- */
/* chooseVelocities on the device state: Maxwell-Boltzmann draws at
 * temperature (kelvin; x 8.314e-7 as equi's rb) from a counter-based
 * generator (splitmix64 of seed, atom, component; uniforms on (0, 1) with
 * 2^32 levels in place of rand()), inverse error function (CUDA erfinv),
 * momentum removal to 1e-15 and rescaling to the temperature.  Kept from the
 * reference: many-body atoms i, i + 1 (i even, i < n_mb) share one draw made
 * with atom i's mass; the momentum sums before the removal count such a pair
 * once, and so does the total mass; the z draw applies the inverse error
 * function before the affine map.  Where the reference's removal loop would
 * never converge (the pairs' second atoms weigh as much as totalm or more,
 * e.g. N-N pairs only), MD_BAD_ARGUMENT. */
md_status md_choose_velocities(md_ctx* ctx, double temperature, unsigned long long seed);
/* equi's schedule (cpu/equi/Host.cpp:174-175): after every step t with
 * t % every == 0 (every = 50 in the reference) new velocities as
 * md_choose_velocities, each from a new stream of seed; every <= 0: off. */
md_status md_set_equilibration(md_ctx* ctx, double temperature, unsigned long long seed,
                               int every);
/* tailResults on the device: pairs i < j of the first n_mb atoms of
 * different species closer than 2 reNO (FP64, the reference's arithmetic),
 * in the reference's order; the first `capacity` pairs into pairs[2k],
 * pairs[2k + 1], their total into *count. */
md_status md_tail_pairs(md_ctx* ctx, int* pairs, int capacity, int* count);

#ifdef __cplusplus
}
#endif
#endif
