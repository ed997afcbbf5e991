// The step engine behind the md_* C ABI (include/mdgb.h).
//
// One context owns one system on one GPU: the Gear state in the reference's
// AoS layouts (real4 positions, real3 vectors, real = double), the LJ and
// bond-order neighbour lists, and the scratch of the force kernels.  md_step
// replays the body of cpu/cpumd/Host.cpp:141-195 on the device:
//   list rebuild when scheduled (readyList + buildList, Host.cpp:143-152)
//   predict -> LJ forces -> bond-order forces -> correct (Host.cpp:155-166)
//   wall hit: forces and a = F/m again (Host.cpp:168-178)
//   record at output steps (performOutput, Host.cpp:181-185)
// Host synchronisation happens only at list builds (the schedule needs the
// largest speed, Host.cpp:289), after a correct in the reference's wall mode
// (the wall flag, as the reference's CUDA host also reads it every step) and
// at the end of md_step.  The periodic mode has no walls and no per-step
// host round trip.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mdgb.h"
#include "md_cluster.h"
#include "md_forces.h"
#include "md_integrate.h"
#include "md_neighbor.cuh"
#include "md_output.h"
#include "md_surrogate.h"

using namespace mdgb;

namespace {

Species species_table(int which) {
  // common/Constants.h:36-43,55-57; the argon table replaces the NG slot
  Species s;
  s.sig[0] = 3.015f;  // NG-N
  s.sig[1] = 2.835f;  // NG-O
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

// cpu/cpumd/Host.cpp:57-61
void list_settings(float rs, float rcut, float& maxnlmove, float& rcutsq) {
  maxnlmove = (rs - rcut) * 0.5f;
  rcutsq = (float)pow((double)rcut, 2);
}

// cpu/cpumd/Host.cpp:289-290; vmax = 0 or an out-of-range quotient is "never"
int next_build(float maxnlmove, double vmax, double dt, int t) {
  double q = ((double)maxnlmove / vmax) / fabs(dt);
  if (!(q < 2147483647.0) || q != q) return 2147483647;
  long long nb = (long long)(int)q + t;
  return nb > 2147483647LL ? 2147483647 : (int)nb;
}

constexpr int kKernels = 8;  // timing ids of md_kernel_time
constexpr long long kSeqTerms = 1LL << 21;  // pair terms per chunk of an in-order record

__global__ void k_begin(md_double4* pos, double* vel, int n, double half_box, int clamp,
                        double vxcm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  md_double4 p = pos[i];
  if (clamp) {
    // cpu/cpumd/Host.cpp:94-104
    if (fabs(p.x) > half_box) p.x = __dmul_rn(half_box, __ddiv_rn(p.x, fabs(p.x)));
    if (fabs(p.y) > half_box) p.y = __dmul_rn(half_box, __ddiv_rn(p.y, fabs(p.y)));
    if (fabs(p.z) > half_box) p.z = __dmul_rn(half_box, __ddiv_rn(p.z, fabs(p.z)));
    pos[i] = p;
  }
  vel[3 * i] = __dadd_rn(vel[3 * i], vxcm);
}

}  // namespace

struct md_ctx {
  md_config cfg{};
  int n = 0;
  std::string err;
  cudaStream_t st = nullptr;
  Species sp{};
  GearCoef gear{};
  double box_size = 0;  // cpu/cpumd/Host.cpp:31, the wall half-width of correct
  float energy_loss = 1.f;
  float lj_maxnlmove = 0, lj_rcutsq = 0, mb_maxnlmove = 0, mb_rcutsq = 0;
  // state
  md_double4* pos = nullptr;
  double *vel = nullptr, *acc = nullptr, *b = nullptr, *c = nullptr, *f3 = nullptr,
         *f3_tmp = nullptr;
  float4* posf = nullptr;
  NeighborList lj, mb;
  // precision form, periodic, LJ only: the cluster kernel; the state is then
  // stored in cell order and cl.orig maps it to the caller's numbering
  bool cluster = false;
  ClusterList cl;
  double* io = nullptr;  // 4 doubles per atom: permuted transfers
  int* inv = nullptr;    // caller's index -> stored position (cell order)
  int inv_version = -1;  // cl.version that inv was computed for
  md_double4* pos_alt = nullptr;  // next positions of the fused force + Gear kernel
  float4* posf_alt = nullptr;
  // independent periodic replicas (batched form): atoms of replica k are
  // [sum of n before k, + n), each in its own box
  bool batch = false;
  std::vector<ClusterReplica> reps_in;
  int* rep_ranges = nullptr;    // device: (first atom, atoms) per replica
  double* rep_buf = nullptr;    // device: 3 energies + 16 record doubles per replica
  // CUDA graphs of a window of fused steps (replayed while nothing else is
  // due): two slots, since a correct-only step swaps the position buffers
  // once and windows then start from either buffer order
  bool graphs = false;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  std::vector<unsigned char> gsig[2];
  int glast = 0;  // slot replayed last
  // learned surrogate of the bond-order term (not owned): used while its
  // force error, measured by the exact kernel every sur_every steps, stays
  // within sur_threshold; otherwise the exact kernel computes the forces
  md_surrogate* sur = nullptr;
  double sur_threshold = 0.0, sur_err = -1.0, sur_err_max = -1.0;
  int sur_every = 10, sur_last_check = -1;
  bool sur_use = false;
  long long sur_steps = 0, sur_exact_steps = 0, sur_checks = 0, sur_rejects = 0;
  // checks declined for descriptors outside the training range (steps
  // declined between checks are counted on the device, sur_flags[1])
  long long sur_declined = 0;
  double *sur_fx = nullptr, *sur_fs = nullptr;  // check buffers (3 doubles per many-body atom)
  // device: [0] this step's "surrogate declined, exact forces" flag, [1] the
  // declined steps between checks (read by md_surrogate_report)
  int* sur_flags = nullptr;
  long long graph_windows = 0;
  // bond-order scratch
  uint32_t* mb_sl = nullptr;
  int* mb_slen = nullptr;
  void *xsi = nullptr, *xsj = nullptr;
  long long mb_elems = 0;
  // flags and reductions
  int* status = nullptr;
  int wait_limit = 1 << 20;  // polls of a bounded mbarrier wait (md_set_wait_limit)
  double* seq_buf = nullptr;  // pair terms of records in the reference's order (2 x kSeqTerms)
  int* wall_flag = nullptr;
  int* missing = nullptr;
  Scratch sc;
  double* epart = nullptr;
  long long epart_cap = 0;
  double* dsc = nullptr;  // device scalars: th8[0..7] elj[8..10] emb[11..13] ref[14..15],
                          // record scratch [16..31], surrogate energy [32]
  double* rec = nullptr;
  int rec_cap = 0, nrec = 0;
  // schedule
  int t = 0, lj_next = 0, mb_next = 0, printout = 0;
  bool begun = false;
  bool predicted = false;  // the state already holds the prediction for step t
  int all_ng = 0;          // every atom is of the NG species (set at upload)
  md_stats stats{};
  // timing
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<int> pending_weight;  // launches each pending interval stands for
  double kt_ms[kKernels] = {};
  long long kt_n[kKernels] = {};

  // animation frames (cpu/cpumd/Host.cpp:83,126,188-192): converted on the
  // device into one of two slots and streamed to pinned host blocks on
  // io_st; a slot is reused only after its copy completed (a stream wait,
  // not a host wait)
  int anim_every = -1, anim_next = 0, anim_frames = 0, anim_slot = 0, anim_per_block = 1;
  float* anim_dev = nullptr;  // 2 slots of 7 floats per atom
  cudaStream_t io_st = nullptr;
  cudaEvent_t anim_ready[2] = {nullptr, nullptr}, anim_done[2] = {nullptr, nullptr};
  bool anim_busy[2] = {false, false};
  std::vector<float*> anim_blocks;  // pinned host memory, anim_per_block frames each
  // equilibration (cpu/equi/Host.cpp:174-175): new Maxwell-Boltzmann
  // velocities after every equi_every-th step
  int equi_every = 0;
  double equi_temp = 0;
  unsigned long long equi_seed = 0, equi_draws = 0;

  bool mixed() const { return cfg.precision == MD_PREC_MIXED; }
  bool permuted() const { return cluster && cl.built; }
  bool walls() const { return !cfg.periodic; }
};

namespace {

md_status fail(md_ctx* c, md_status s, const std::string& msg) {
  c->err = msg;
  return s;
}

md_status cuda_fail(md_ctx* c, cudaError_t e, const char* where) {
  c->err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? MD_OUT_OF_MEMORY : MD_CUDA_ERROR;
}

#define CK(expr, where)                                  \
  do {                                                   \
    cudaError_t e_ = (expr);                             \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, where); \
  } while (0)

cudaEvent_t take_event(md_ctx* c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

struct Timed {
  md_ctx* c;
  int id;
  int weight;
  cudaEvent_t a = nullptr, b = nullptr;
  Timed(md_ctx* c_, int id_, int weight_ = 1) : c(c_), id(id_), weight(weight_) {
    if (c->timing) {
      a = take_event(c);
      b = take_event(c);
      cudaEventRecord(a, c->st);
    }
  }
  ~Timed() {
    if (c->timing) {
      cudaEventRecord(b, c->st);
      c->pending.push_back({id, {a, b}});
      c->pending_weight.push_back(weight);
    }
  }
};

void resolve_timing(md_ctx* c) {
  for (size_t k = 0; k < c->pending.size(); k++) {
    auto& p = c->pending[k];
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
      c->kt_ms[p.first] += ms;
      c->kt_n[p.first] += c->pending_weight[k];
    }
    c->ev_pool.push_back(p.second.first);
    c->ev_pool.push_back(p.second.second);
  }
  c->pending.clear();
  c->pending_weight.clear();
}

md_status ensure_epart(md_ctx* c, long long need) {
  if (need <= c->epart_cap) return MD_OK;
  if (c->epart) cudaFree(c->epart);
  c->epart = nullptr;
  CK(cudaMalloc(&c->epart, sizeof(double) * (size_t)need), "epart");
  c->epart_cap = need;
  return MD_OK;
}

md_status ensure_mb_scratch(md_ctx* c) {
  long long need = (long long)c->mb.cap * (c->cfg.n_mb > 0 ? c->cfg.n_mb : 1);
  if (need <= c->mb_elems && c->mb_sl) return MD_OK;
  for (void** p : {(void**)&c->mb_sl, &c->xsi, &c->xsj})
    if (*p) {
      cudaFree(*p);
      *p = nullptr;
    }
  size_t es = sizeof(double);
  CK(cudaMalloc(&c->mb_sl, sizeof(uint32_t) * (size_t)need), "mb short list");
  CK(cudaMalloc(&c->xsi, es * (size_t)need), "mb xi");
  CK(cudaMalloc(&c->xsj, es * (size_t)need), "mb xi");
  c->mb_elems = need;
  return MD_OK;
}

ForceArgs lj_args(md_ctx* c, double* f3, double* epart) {
  ForceArgs a;
  a.pos = c->pos;
  a.posf = c->posf;
  a.f3 = f3;
  a.n = c->n;
  a.list = c->lj.list;
  a.len = c->lj.len;
  a.ld = c->lj.ld;
  a.tmap = c->lj.tmap_ok ? &c->lj.tmap : nullptr;
  a.all_ng = c->all_ng;
  a.status = c->status;
  a.walker = make_walker(c->lj);
  a.skin = c->lj.skin;
  a.parity = c->t & 1;
  a.cap = c->lj.cap;
  a.rv2 = c->lj.rv2_keep;
  a.pos_build = c->lj.pos_build;
  a.rcutsq = (double)c->lj_rcutsq;
  a.sp = c->sp;
  a.epart = epart;
  a.wait_limit = c->wait_limit;
  return a;
}

MbArgs mb_args(md_ctx* c, double* f3, int ljexist) {
  MbArgs a;
  a.pos = c->pos;
  a.posf = c->posf;
  a.f3 = f3;
  a.n = c->cfg.n_mb;
  a.list = c->mb.list;
  a.len = c->mb.len;
  a.ld = c->mb.ld;
  a.grid = c->mb.grid;
  a.cell3 = c->mb.cell3;
  a.ref_rows = nullptr;
  a.ref_nls = 0;
  a.ref_nlargest = 0;
  a.rcutsq = (double)c->mb_rcutsq;
  a.ljexist = ljexist;
  a.sl = c->mb_sl;
  a.slen = c->mb_slen;
  a.xsi = c->xsi;
  a.xsj = c->xsj;
  a.missing = c->missing;
  a.epart1 = nullptr;
  a.epart2 = nullptr;
  return a;
}

// Host.cpp:132-135 / :157-161: LJ over all atoms (overwrites), bond order
// over the first n_mb atoms (accumulates when LJ is on).
// replicas of the cluster structure: the batch's, or the one periodic box
std::vector<ClusterReplica> cluster_reps(const md_ctx* c) {
  if (c->batch) return c->reps_in;
  std::vector<ClusterReplica> reps(1);
  memset(reps.data(), 0, sizeof(ClusterReplica));
  reps[0].n = c->n;
  reps[0].L = c->cfg.box;
  return reps;
}

ClusterForceArgs cl_args(md_ctx* c, double* f3, double* epart) {
  ClusterForceArgs a;
  a.cl = &c->cl;
  a.posf = c->posf;
  a.pos = c->pos;
  a.f3 = f3;
  a.step = c->t;
  a.rcutsq = (double)c->lj_rcutsq;
  a.sp = c->sp;
  a.all_ng = c->all_ng;
  a.epart = epart;
  a.status = c->status;
  a.gear = nullptr;
  a.wait_limit = c->wait_limit;
  return a;
}

// bond-order forces of the step: exact, or the surrogate's (checked against
// the exact kernel every sur_every steps)
md_status mb_forces_step(md_ctx* c, double* f3) {
  const int nmb = c->cfg.n_mb;
  const int acc = c->cfg.use_lj;
  if (c->t - c->sur_last_check >= c->sur_every || c->sur_last_check < 0 || c->t < c->sur_last_check) {
    MbArgs a = mb_args(c, c->sur_fx, 0);
    launch_mb(a, c->mixed(), false, c->st);
    bool declined = false;
    int r = sur_forces(*c->sur, c->pos, nmb, make_walker(c->mb), c->sur_fs, 0, nullptr, c->status,
                       c->st, &declined);
    if (r) return r == -1 ? fail(c, MD_BAD_ARGUMENT, "surrogate not trained")
                          : cuda_fail(c, (cudaError_t)r, "surrogate forces");
    // an atom outside the training data's descriptor range fails the check
    double err = INFINITY;
    if (!declined) {
      r = sur_rel_err(c->sur_fs, c->sur_fx, nmb, c->sur->scratch, &err, c->st);
      if (r) return cuda_fail(c, (cudaError_t)r, "surrogate check");
      c->sur_err = err;
      c->sur_err_max = std::max(c->sur_err_max, err);
    } else {
      c->sur_declined++;
    }
    c->sur_use = err <= c->sur_threshold;
    c->sur_last_check = c->t;
    c->sur_checks++;
    if (!c->sur_use) c->sur_rejects++;
    c->stats.launches += 12;
  }
  if (c->sur_use) {
    // no host wait: the store of the network's forces and the exact kernels
    // that take the step instead both read the device flag of the range check
    int r = sur_forces(*c->sur, c->pos, nmb, make_walker(c->mb), f3, acc, nullptr, c->status,
                       c->st, nullptr, c->sur_flags, c->sur_flags + 1);
    if (r) return cuda_fail(c, (cudaError_t)r, "surrogate forces");
    MbArgs a = mb_args(c, f3, acc);
    a.run_if = c->sur_flags;
    launch_mb(a, c->mixed(), false, c->st);
    c->stats.launches += 10;
    c->sur_steps++;
  } else {
    launch_mb(mb_args(c, f3, acc), c->mixed(), false, c->st);
    c->sur_exact_steps++;
    c->stats.launches += 3;
  }
  return MD_OK;
}

md_status forces(md_ctx* c, double* f3, bool step = false) {
  if (c->cfg.use_lj) {
    Timed tm(c, 0);
    if (c->cluster)
      launch_lj_cluster(cl_args(c, f3, nullptr), false, c->st);
    else
      launch_lj(lj_args(c, f3, nullptr), c->mixed(), false, c->st);
    c->stats.launches++;
  }
  if (c->cfg.use_mb && c->cfg.n_mb > 0) {
    Timed tm(c, 1);
    if (step && c->sur) return mb_forces_step(c, f3);
    launch_mb(mb_args(c, f3, c->cfg.use_lj), c->mixed(), false, c->st);
    c->stats.launches += 3;
  }
  return MD_OK;
}

GearArgs gear_args(md_ctx* c, int parity) {
  GearArgs g;
  g.pos = c->pos;
  g.vel = c->vel;
  g.acc = c->acc;
  g.b = c->b;
  g.c = c->c;
  g.f3 = c->f3;
  g.n = c->n;
  g.k = c->gear;
  g.sp = c->sp;
  g.posf = c->mixed() ? c->posf : nullptr;
  const float4* pb = c->cluster ? c->cl.pos_build : (c->lj.compact ? c->lj.pos_build : nullptr);
  const double trip = c->cluster ? c->cl.trip_dist : c->lj.trip_dist;
  int* skinf = c->cluster ? c->cl.skin : c->lj.skin;
  const bool skin = c->cfg.use_lj && pb;
  g.pos_build = skin ? pb : nullptr;
  g.trip2 = skin ? (float)(trip * trip) : 0.f;
  if (skin && trip <= 0) g.trip2 = -1.f;  // skin too thin: always walk full rows
  g.trip = skin ? skinf + (c->cluster ? parity % 3 : parity & 1) : nullptr;
  g.status = c->status;
  g.exact = !c->mixed();
  for (int k = 0; k < 3; k++) g.inv_mass[k] = 1.0 / (double)c->sp.mass[k];
  g.npos = c->box_size;
  g.energy_loss = c->energy_loss;
  g.walls = c->walls();
  g.wall_flag = c->wall_flag;
  return g;
}

md_status check_status(md_ctx* c) {
  int s = 0;
  CK(cudaMemcpyAsync(&s, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->st), "status");
  int miss = 0;
  CK(cudaMemcpyAsync(&miss, c->missing, sizeof(int), cudaMemcpyDeviceToHost, c->st), "status");
  CK(cudaStreamSynchronize(c->st), "step");
  CK(cudaGetLastError(), "step");
  c->stats.missing_xi = miss;
  if (s & ST_NONFINITE) return fail(c, MD_NONFINITE, "non-finite position or velocity");
  if (s & ST_CELL_OVERFLOW) return fail(c, MD_CELL_OVERFLOW, "cell grid out of range");
  if (s & ST_TMA_TIMEOUT) return fail(c, MD_TIMEOUT, "a TMA transfer did not complete in time");
  return MD_OK;
}

// The cluster build put the state in its cell order: back to the caller's
// numbering, and the row-list kernel takes over from here on.
void leave_cluster(md_ctx* c) {
  launch_unpermute((const double*)c->pos, (double*)c->pos_alt, c->cl.orig, c->n, 4, c->st);
  std::swap(c->pos, c->pos_alt);
  double** v3[5] = {&c->vel, &c->acc, &c->b, &c->c, &c->f3};
  for (int k = 0; k < 5; k++)
    if (*v3[k] && c->cl.v3_tmp[k]) {
      launch_unpermute(*v3[k], c->cl.v3_tmp[k], c->cl.orig, c->n, 3, c->st);
      std::swap(*v3[k], c->cl.v3_tmp[k]);
    }
  c->stats.launches += 6;
  c->cluster = false;
  c->graphs = false;
  c->predicted = false;
  c->stats.lj_cluster = 0;
}

// readyList + buildList for the lists due at step t (Host.cpp:143-152)
md_status rebuild(md_ctx* c, int t) {
  Timed tm(c, 4);
  unsigned long long um[2];
  launch_ready(c->pos, c->vel, c->n, c->sc.umax, c->status, c->st);
  CK(cudaMemcpyAsync(um, c->sc.umax, sizeof(um), cudaMemcpyDeviceToHost, c->st), "ready");
  int s = 0;
  CK(cudaMemcpyAsync(&s, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->st), "ready");
  CK(cudaStreamSynchronize(c->st), "ready");
  c->stats.launches += 1;
  if (s & ST_NONFINITE) return fail(c, MD_NONFINITE, "non-finite position or velocity");
  double vmax, maxabs;
  memcpy(&vmax, &um[0], 8);
  memcpy(&maxabs, &um[1], 8);
  const double box_list = maxabs * 2;
  const bool both = c->cfg.periodic != 0;
  const double dt = (double)c->cfg.dt;
  bool did_lj = false;
  if (c->cluster && c->cfg.use_lj && (c->lj_next == t || both)) {
    if (c->cl.skin) {
      int sk[5];
      CK(cudaMemcpy(sk, c->cl.skin, sizeof(sk), cudaMemcpyDeviceToHost), "skin");
      c->stats.list_trips += sk[4];
      if (sk[3]) c->cl.headroom *= 1.5f;  // a refreshed row did not fit: more room
      CK(cudaMemsetAsync(c->cl.skin + 4, 0, sizeof(int), c->st), "skin");
    }
    CK(cudaMemsetAsync(c->status, 0, sizeof(int), c->st), "status");
    std::vector<ClusterReplica> reps = cluster_reps(c);
    double** v3[5] = {&c->vel, &c->acc, &c->b, &c->c, &c->f3};
    std::string e;
    int r = cluster_build(c->cl, reps, c->cfg.lj_rs, sqrt((double)c->lj_rcutsq), &c->pos, v3,
                          c->posf, c->sc, c->status, c->st, e);
    c->stats.launches += 17;
    if (r == -1 && c->cfg.lj_kernel == MD_LJ_AUTO && !c->batch &&
        e.find("shared-memory stage") != std::string::npos) {
      // a neighbourhood too dense for the staged shared memory: the row-list
      // kernel takes over (the state goes back to the caller's numbering)
      leave_cluster(c);  // the row-list build below runs instead
    } else {
      if (r != 0) {
        if (r == -1) return fail(c, e.find("non-finite") != std::string::npos ? MD_NONFINITE : MD_BAD_CONFIG, e);
        return cuda_fail(c, (cudaError_t)r, "LJ cluster build");
      }
      c->lj_next = next_build(c->lj_maxnlmove, vmax, dt, t);
      c->stats.list_builds++;
      c->stats.lj_max_row = c->cl.maxlen;
      c->stats.lj_nlargest = 0;
      c->stats.lj_cells = c->cl.h_rep[0].G;
      c->stats.lj_list_entries = c->cl.entries;
      c->stats.lj_tma = 0;
      c->stats.lj_cluster = 1;
      c->stats.cluster_segments = c->cl.nseg;
      c->stats.cluster_max_staged = c->cl.max_staged;
      return MD_OK;
    }
  }
  if (c->cfg.use_lj && (c->lj_next == t || both)) {
    if (c->lj.skin) {
      int sk[4];
      CK(cudaMemcpy(sk, c->lj.skin, sizeof(sk), cudaMemcpyDeviceToHost), "skin");
      c->stats.list_trips += sk[3];
      if (sk[2]) c->lj.headroom *= 1.5f;  // a refreshed row did not fit: more room
      CK(cudaMemsetAsync(c->lj.skin + 3, 0, sizeof(int), c->st), "skin");
    }
    CK(cudaMemsetAsync(c->status, 0, sizeof(int), c->st), "status");
    Grid g = c->cfg.periodic ? make_grid_periodic(c->cfg.box, c->cfg.lj_rs)
                             : make_grid_reference(box_list, c->cfg.lj_rs);
    std::string e;
    int r = list_build(c->lj, c->pos, c->n, g, 1, c->cfg.lj_rs, sqrt((double)c->lj_rcutsq),
                       c->sc, c->status, c->st, e);
    c->stats.launches += 9;
    if (r != 0) {
      if (r == -1) return fail(c, e.find("non-finite") != std::string::npos ? MD_NONFINITE : MD_CELL_OVERFLOW, e);
      return cuda_fail(c, (cudaError_t)r, "LJ list build");
    }
    c->lj_next = next_build(c->lj_maxnlmove, vmax, dt, t);
    c->stats.list_builds++;
    c->stats.lj_max_row = c->lj.max_len;
    c->stats.lj_nlargest = c->lj.nlargest;
    c->stats.lj_cells = c->lj.grid.cells;
    c->stats.lj_list_entries = c->lj.entries;
    c->stats.lj_tma = c->lj.tmap_ok;
    did_lj = true;
  }
  if (c->cfg.use_mb && c->cfg.n_mb > 0 && (c->mb_next == t || both)) {
    Grid g = c->cfg.periodic ? make_grid_periodic(c->cfg.box, c->cfg.mb_rs)
                             : make_grid_reference(box_list, c->cfg.mb_rs);
    std::string e;
    if (!did_lj) CK(cudaMemsetAsync(c->status, 0, sizeof(int), c->st), "status");
    int r = list_build(c->mb, c->pos, c->cfg.n_mb, g, 0, 0.f, sqrt((double)c->mb_rcutsq), c->sc,
                       c->status, c->st, e);
    c->stats.launches += 9;
    if (r != 0) {
      if (r == -1) return fail(c, e.find("non-finite") != std::string::npos ? MD_NONFINITE : MD_CELL_OVERFLOW, e);
      return cuda_fail(c, (cudaError_t)r, "many-body list build");
    }
    if (!c->mb_slen) CK(cudaMalloc(&c->mb_slen, sizeof(int) * (size_t)c->cfg.n_mb), "mb slen");
    md_status ms = ensure_mb_scratch(c);
    if (ms != MD_OK) return ms;
    c->mb_next = next_build(c->mb_maxnlmove, vmax, dt, t);
    c->stats.list_builds++;
    c->stats.mb_nlargest = c->mb.nlargest;
    c->stats.mb_cells = c->mb.grid.cells;
  }
  if (both) {
    // periodic box: both lists are rebuilt together (positions wrap at a build)
    int m = 2147483647;
    if (c->cfg.use_lj && c->lj_next < m) m = c->lj_next;
    if (c->cfg.use_mb && c->mb_next < m) m = c->mb_next;
    if (c->cfg.use_lj) c->lj_next = m;
    if (c->cfg.use_mb) c->mb_next = m;
  }
  if (c->mixed()) {
    launch_posf(c->pos, c->posf, c->n, c->st);
    c->stats.launches++;
  }
  return MD_OK;
}

}  // namespace
extern "C" md_status ensure_inv(md_ctx* c);
namespace {

// thermo + energies of the current state into a 16-double record at rec16
md_status make_record(md_ctx* c, int t, double* rec16) {
  double* th8 = c->dsc;
  double* elj = c->dsc + 8;
  double* emb = c->dsc + 11;
  double* ref = c->dsc + 14;
  const bool seq = c->cfg.reference_energy == 2;  // the reference's summation order
  const int* inv = nullptr;
  if (seq && c->permuted()) {
    md_status s = ensure_inv(c);
    if (s != MD_OK) return s;
    inv = c->inv;
  }
  if (seq) {
    launch_thermo_seq(c->pos, c->vel, inv, c->n, c->sp, th8, c->st);
    c->stats.launches += 1;
  } else {
    launch_thermo(c->pos, c->vel, c->n, c->sp, c->sc.dpart, th8, c->st);
    c->stats.launches += 5;
  }
  CK(cudaMemsetAsync(elj, 0, sizeof(double) * 8, c->st), "record");
  if (c->cfg.use_lj) {
    int B = c->cluster ? cluster_blocks(c->cl) : lj_blocks(c->n);
    md_status s = ensure_epart(c, 3LL * B);
    if (s != MD_OK) return s;
    if (c->cluster)
      launch_lj_cluster(cl_args(c, c->f3_tmp, c->epart), true, c->st);
    else
      launch_lj(lj_args(c, c->f3_tmp, c->epart), c->mixed(), true, c->st);
    launch_sum_partials(c->epart, B, 3, elj, c->st);
    c->stats.launches += 2;
  }
  if (c->cfg.use_mb && c->cfg.n_mb > 0) {
    int B = mb_blocks(c->cfg.n_mb);
    md_status s = ensure_epart(c, 3LL * B);
    if (s != MD_OK) return s;
    MbArgs a = mb_args(c, c->f3_tmp, 0);
    a.epart1 = c->epart;
    a.epart2 = c->epart + 2LL * B;
    launch_mb(a, c->mixed(), true, c->st);
    launch_sum_partials(a.epart1, B, 2, emb, c->st);
    launch_sum_partials(a.epart2, B, 1, emb + 2, c->st);
    c->stats.launches += 5;
  }
  if (seq) {
    if (!c->seq_buf) CK(cudaMalloc(&c->seq_buf, sizeof(double) * 2 * (size_t)kSeqTerms),
                        "record terms");
    c->stats.launches +=
        launch_ref_potential_seq(c->pos, inv, c->n, c->sp, c->seq_buf, kSeqTerms, ref, c->st);
  } else if (c->cfg.reference_energy) {
    md_status s = ensure_epart(c, 2LL * c->n);
    if (s != MD_OK) return s;
    launch_ref_potential(c->pos, c->n, c->sp, c->epart, ref, c->st);
    c->stats.launches += 2;
  }
  launch_record(th8, elj, emb, ref, c->cfg.reference_energy, (double)t * (double)c->cfg.dt,
                (double)t, rec16, c->st);
  c->stats.launches++;
  return MD_OK;
}

md_status push_record(md_ctx* c, int t) {
  if (c->nrec >= c->rec_cap) {
    int cap = c->rec_cap ? 2 * c->rec_cap : 64;
    double* nr = nullptr;
    CK(cudaMalloc(&nr, sizeof(double) * 16 * (size_t)cap), "records");
    if (c->rec) {
      CK(cudaMemcpyAsync(nr, c->rec, sizeof(double) * 16 * (size_t)c->nrec,
                         cudaMemcpyDeviceToDevice, c->st), "records");
      CK(cudaStreamSynchronize(c->st), "records");
      cudaFree(c->rec);
    }
    c->rec = nr;
    c->rec_cap = cap;
  }
  md_status s = make_record(c, t, c->rec + 16 * (size_t)c->nrec);
  if (s == MD_OK) c->nrec++;
  return s;
}

// One animation frame of the current state (pushAnim, common/Results.cpp:12-31).
md_status capture_frame(md_ctx* c) {
  const size_t per = 7 * (size_t)c->n;
  const size_t fb = sizeof(float) * per;
  const int s = c->anim_slot;
  c->anim_slot ^= 1;
  if (c->anim_busy[s]) CK(cudaStreamWaitEvent(c->st, c->anim_done[s], 0), "animation");
  float* slot = c->anim_dev + (size_t)s * per;
  launch_anim_pack(c->pos, c->vel, c->permuted() ? c->cl.orig : nullptr, c->n, slot, c->st);
  c->stats.launches++;
  CK(cudaEventRecord(c->anim_ready[s], c->st), "animation");
  const size_t blk = (size_t)(c->anim_frames / c->anim_per_block);
  while (c->anim_blocks.size() <= blk) {
    float* h = nullptr;
    CK(cudaHostAlloc((void**)&h, fb * (size_t)c->anim_per_block, cudaHostAllocDefault),
       "animation frames");
    c->anim_blocks.push_back(h);
  }
  float* host = c->anim_blocks[blk] + (size_t)(c->anim_frames % c->anim_per_block) * per;
  CK(cudaStreamWaitEvent(c->io_st, c->anim_ready[s], 0), "animation");
  CK(cudaMemcpyAsync(host, slot, fb, cudaMemcpyDeviceToHost, c->io_st), "animation");
  CK(cudaEventRecord(c->anim_done[s], c->io_st), "animation");
  c->anim_busy[s] = true;
  c->anim_frames++;
  return MD_OK;
}

bool anim_due(const md_ctx* c, int t) { return c->anim_every >= 0 && c->anim_next == t; }

bool equi_due(const md_ctx* c, int t) { return c->equi_every > 0 && t % c->equi_every == 0; }

// chooseVelocities (cpu/equi/Host.cpp:416-572) on the current state;
// temperature in kelvin (times rb = 8.314e-7, :85-86)
md_status choose_velocities(md_ctx* c, double temperature, unsigned long long seed) {
  int it = 0;
  const int r = equi_velocities(c->pos, c->vel, c->permuted() ? c->cl.orig : nullptr, c->n,
                                c->cfg.n_mb, c->sp, temperature * 8.314e-7, seed, c->sc.dpart,
                                &it, c->st);
  c->stats.launches += 2 * it + 6;
  if (r == -1)
    return fail(c, MD_BAD_ARGUMENT,
                "momentum removal does not converge: the many-body pairs enter the total mass "
                "once (cpu/equi/Host.cpp:474-478), so each shift overshoots at least as far "
                "as it corrects");
  if (r) return cuda_fail(c, (cudaError_t)r, "choose velocities");
  return MD_OK;
}

bool due(const md_ctx* c, int t) {
  return (c->cfg.use_lj && c->lj_next == t) || (c->cfg.use_mb && c->mb_next == t);
}

// Forces of step t, correct of step t and predict of step t + 1 in one
// kernel (cluster path); the next positions go to the other buffer.  With
// predict false the kernel stops after the correct and also stores the forces
// in f3: the other buffer then holds the corrected state of step t.
void launch_fused(md_ctx* c, bool predict = true) {
  GearArgs g = gear_args(c, c->t + 1);
  ClusterGearArgs cg;
  cg.pos_next = c->pos_alt;
  cg.posf_next = c->posf_alt;
  cg.vel = c->vel;
  cg.acc = c->acc;
  cg.b = c->b;
  cg.c = c->c;
  cg.k = c->gear;
  for (int k = 0; k < 3; k++) cg.inv_mass[k] = g.inv_mass[k];
  cg.trip2 = g.trip2;
  cg.correct_only = !predict;
  ClusterForceArgs a = cl_args(c, predict ? nullptr : c->f3, nullptr);
  a.gear = &cg;
  launch_lj_cluster(a, false, c->st);
}

void advance_fused(md_ctx* c) {
  std::swap(c->pos, c->pos_alt);
  std::swap(c->posf, c->posf_alt);
  c->predicted = true;
  c->stats.launches++;
  c->t++;
  c->stats.steps++;
}

// A window of kGraphSteps fused steps replayed as one CUDA graph.  The
// window starts at step t with the prediction in place and needs no list
// build, record or call boundary inside.  The graph is captured again only
// when anything it bakes in changed (buffers after a list build, tiles, the
// step's phase in the 3-step rotation of the skin flags).
constexpr int kGraphSteps = 6;  // even (buffers return to place) and a multiple of 3

bool window_ok(const md_ctx* c, int s, int nsteps) {
  if (!c->cluster || !c->graphs || !c->predicted) return false;
  if (s + kGraphSteps > nsteps - 1) return false;  // the call's last step is not fused
  const int t = c->t;
  for (int u = 0; u < kGraphSteps; u++) {
    if (c->cfg.output_timesteps > 0 && c->printout == t + u) return false;
    if (anim_due(c, t + u)) return false;
    if (equi_due(c, t + u)) return false;
    if (due(c, t + u + 1)) return false;
  }
  return true;
}

md_status run_window(md_ctx* c) {
  struct Sig {
    int t6, nseg, max_staged, block, all_ng, cap, ld, wait_limit, row_loads, grouped;
    float trip2;
    const void* ptr[14];
    unsigned char rmap[sizeof(CUtensorMap)];
  } sig;
  memset(&sig, 0, sizeof(sig));
  sig.t6 = c->t % kGraphSteps;
  sig.nseg = c->cl.nseg;
  sig.max_staged = c->cl.max_staged;
  sig.block = c->cl.block;
  sig.all_ng = c->all_ng;
  sig.cap = c->cl.cap;
  sig.ld = c->cl.ld;
  sig.wait_limit = c->wait_limit;
  sig.row_loads = c->cl.row_loads;
  sig.grouped = c->cl.grouped;
  sig.trip2 = gear_args(c, c->t + 1).trip2;
  const void* ptrs[14] = {c->pos, c->pos_alt, c->posf, c->posf_alt, c->vel, c->acc, c->b, c->c,
                          c->cl.seg, c->cl.rows, c->cl.len, c->cl.pos_build, c->cl.skin,
                          c->cl.rep};
  memcpy(sig.ptr, ptrs, sizeof(ptrs));
  memcpy(sig.rmap, &c->cl.rmap, sizeof(CUtensorMap));
  const unsigned char* sb = (const unsigned char*)&sig;
  int slot = -1;
  for (int k = 0; k < 2; k++)
    if (c->gexec[k] && c->gsig[k].size() == sizeof(sig) &&
        memcmp(c->gsig[k].data(), sb, sizeof(sig)) == 0)
      slot = k;
  if (slot < 0) {
    slot = c->gexec[c->glast] ? 1 - c->glast : c->glast;  // the slot not replayed last
    // capture the window's launches (the host state is restored afterwards)
    const int t0 = c->t;
    const md_stats st0 = c->stats;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal), "graph capture");
    for (int u = 0; u < kGraphSteps; u++) {
      launch_fused(c);
      advance_fused(c);
    }
    cudaError_t e = cudaStreamEndCapture(c->st, &g);
    c->t = t0;
    c->stats = st0;  // kGraphSteps swaps: buffers are back in place
    if (e != cudaSuccess) return cuda_fail(c, e, "graph capture");
    cudaGraphExec_t& x = c->gexec[slot];
    bool updated = false;
    if (x) {
      cudaGraphExecUpdateResultInfo info;
      updated = cudaGraphExecUpdate(x, g, &info) == cudaSuccess;
      if (!updated) {
        cudaGetLastError();
        cudaGraphExecDestroy(x);
        x = nullptr;
      }
    }
    if (!updated) {
      e = cudaGraphInstantiate(&x, g, 0);
      if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        x = nullptr;
        c->gsig[slot].clear();
        return cuda_fail(c, e, "graph instantiate");
      }
    }
    cudaGraphDestroy(g);
    c->gsig[slot].assign(sb, sb + sizeof(sig));
  }
  c->glast = slot;
  {
    Timed tm(c, 6, kGraphSteps);
    CK(cudaGraphLaunch(c->gexec[slot], c->st), "graph launch");
  }
  for (int u = 0; u < kGraphSteps; u++) advance_fused(c);
  c->graph_windows++;
  return MD_OK;
}

// One iteration of cpu/cpumd/Host.cpp:141-195.  In the precision form with a
// periodic box, correct(t) and predict(t+1) run as one kernel unless step
// t+1 rebuilds a list, step t records output, or this is the last step of
// the call (the state between calls is always the corrected one).
md_status step_once(md_ctx* c, bool last) {
  const int t = c->t;
  if (due(c, t)) {
    md_status s = rebuild(c, t);
    if (s != MD_OK) return s;
  }
  if (!c->predicted) {
    GearArgs g = gear_args(c, t);
    Timed tm(c, 2);
    launch_predict(g, c->st);
    c->stats.launches++;
  }
  c->predicted = false;
  const bool output = c->cfg.output_timesteps > 0 && c->printout == t;
  const bool anim = anim_due(c, t);
  const bool equi = equi_due(c, t);
  const bool fuse =
      c->mixed() && !c->walls() && !last && !output && !anim && !equi && !due(c, t + 1);
  if (c->cluster && fuse) {
    {
      Timed tm(c, 6);
      launch_fused(c);
    }
    advance_fused(c);
    return MD_OK;
  }
  if (c->cluster) {
    // forces and correct of step t in one kernel, without the predict (a list
    // build, a record, a frame, new velocities or the call's end follows)
    {
      Timed tm(c, 7);
      launch_fused(c, false);
    }
    std::swap(c->pos, c->pos_alt);
    std::swap(c->posf, c->posf_alt);
    c->stats.launches++;
  } else {
    {
      md_status fs = forces(c, c->f3, true);
      if (fs != MD_OK) return fs;
    }
    if (c->walls()) CK(cudaMemsetAsync(c->wall_flag, 0, sizeof(int), c->st), "wall flag");
    {
      Timed tm(c, 3);
      if (fuse) {
        launch_correct_predict(gear_args(c, t + 1), c->st);
        c->predicted = true;
      } else {
        launch_correct(gear_args(c, t), c->st);
      }
      c->stats.launches++;
    }
  }
  if (c->walls()) {
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, c->wall_flag, sizeof(int), cudaMemcpyDeviceToHost, c->st), "wall");
    CK(cudaStreamSynchronize(c->st), "wall");
    if (flag) {
      c->stats.wall_hits++;
      forces(c, c->f3);
      launch_accel(c->pos, c->acc, c->f3, c->n, c->sp, c->st);
      c->stats.launches++;
    }
  }
  if (output) {
    md_status s = push_record(c, t);
    if (s != MD_OK) return s;
    c->printout += c->cfg.output_timesteps;
  }
  if (anim) {
    md_status s = capture_frame(c);
    if (s != MD_OK) return s;
    c->anim_next += c->anim_every;
  }
  if (equi) {
    // a new stream of draws for every reassignment
    md_status s = choose_velocities(c, c->equi_temp, c->equi_seed + 0x632BE59BD9B4E019ull *
                                                                      ++c->equi_draws);
    if (s != MD_OK) return s;
  }
  c->t++;
  c->stats.steps++;
  return MD_OK;
}

}  // namespace

extern "C" {

const char* md_status_string(md_status s) {
  switch (s) {
    case MD_OK: return "ok";
    case MD_BAD_CONFIG: return "bad configuration";
    case MD_LIST_OVERFLOW: return "neighbour list does not fit the buffer";
    case MD_NONFINITE: return "non-finite value";
    case MD_TIMEOUT: return "device wait timed out";
    case MD_CUDA_ERROR: return "CUDA error";
    case MD_BAD_ARGUMENT: return "bad argument";
    case MD_NO_DEVICE: return "no CUDA device";
    case MD_OUT_OF_MEMORY: return "out of device memory";
    case MD_CELL_OVERFLOW: return "cell grid out of range";
  }
  return "unknown status";
}

const char* md_last_error(const md_ctx* c) { return c ? c->err.c_str() : "no context"; }

md_status md_create(const md_config* cfg, md_ctx** out) {
  if (!cfg || !out) return MD_BAD_ARGUMENT;
  *out = nullptr;
  const long long n = (long long)cfg->n_lj + cfg->n_mb;
  if (cfg->n_lj < 0 || cfg->n_mb < 0 || n < 1 || n > kMaxAtoms) return MD_BAD_CONFIG;
  if (!(cfg->dt == cfg->dt) || cfg->dt == 0.f) return MD_BAD_CONFIG;
  if (cfg->use_lj && !(cfg->lj_rcut > 0.f && cfg->lj_rs > cfg->lj_rcut)) return MD_BAD_CONFIG;
  if (cfg->use_mb && !(cfg->mb_rcut > 0.f && cfg->mb_rs >= cfg->mb_rcut &&
                       cfg->mb_rcut < MD_CUTOFF_RIJ))
    return MD_BAD_CONFIG;
  if (cfg->precision != MD_PREC_FP64 && cfg->precision != MD_PREC_MIXED) return MD_BAD_CONFIG;
  if (cfg->species != MD_SPECIES_NEON && cfg->species != MD_SPECIES_ARGON) return MD_BAD_CONFIG;
  if (cfg->periodic) {
    double rsmax = 0;
    if (cfg->use_lj) rsmax = fmax(rsmax, cfg->lj_rs);
    if (cfg->use_mb) rsmax = fmax(rsmax, cfg->mb_rs);
    if (!(cfg->box > 2.0 * rsmax)) return MD_BAD_CONFIG;
    // the bond-order third-body pass needs distinct stencil cells
    if (cfg->use_mb && floor(cfg->box / (double)cfg->mb_rs) < 3) return MD_BAD_CONFIG;
  }
  const bool cluster_ok = cfg->precision == MD_PREC_MIXED && cfg->periodic && cfg->use_lj &&
                          !(cfg->use_mb && cfg->n_mb > 0);
  if (cfg->lj_kernel < MD_LJ_AUTO || cfg->lj_kernel > MD_LJ_CLUSTER) return MD_BAD_CONFIG;
  if (cfg->lj_kernel == MD_LJ_CLUSTER && !cluster_ok) return MD_BAD_CONFIG;
  if (cfg->cluster_cells < 0 || cfg->cluster_cells > kClusterMaxZ) return MD_BAD_CONFIG;
  if (cfg->cluster_threads < 0 || cfg->cluster_threads > 224 || cfg->cluster_threads % 32)
    return MD_BAD_CONFIG;
  if (cfg->cluster_row_loads < 0 || cfg->cluster_row_loads > 4) return MD_BAD_CONFIG;
  if (cfg->cluster_stage_cap != 0 &&
      (cfg->cluster_stage_cap < 64 || cfg->cluster_stage_cap > kClusterMaxStaged))
    return MD_BAD_CONFIG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device || cfg->device < 0)
    return MD_NO_DEVICE;
  md_ctx* c = new md_ctx();
  c->cfg = *cfg;
  c->cluster = cluster_ok && cfg->lj_kernel != MD_LJ_ROWS;
  c->graphs = c->cluster;
  if (cfg->cluster_cells > 0) c->cl.Z = cfg->cluster_cells;
  if (cfg->cluster_threads > 0) c->cl.block = cfg->cluster_threads;
  if (cfg->cluster_row_loads > 0) c->cl.row_loads = cfg->cluster_row_loads;
  if (cfg->cluster_stage_cap > 0) c->cl.stage_cap = cfg->cluster_stage_cap;
  c->n = (int)n;
  c->sp = species_table(cfg->species);
  c->gear = gear_coef((double)cfg->dt);
  c->box_size = pow((double)n, 1.0 / 3.0) * 52.8;  // Host.cpp:31
  c->energy_loss = sqrtf(cfg->energy_loss);        // Host.cpp:73
  if (cfg->use_lj) list_settings(cfg->lj_rs, cfg->lj_rcut, c->lj_maxnlmove, c->lj_rcutsq);
  if (cfg->use_mb) list_settings(cfg->mb_rs, cfg->mb_rcut, c->mb_maxnlmove, c->mb_rcutsq);
  auto bail = [&](cudaError_t e, const char* w) {
    md_status s = cuda_fail(c, e, w);
    md_destroy(c);
    return s;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(cfg->device)) != cudaSuccess) return bail(e, "cudaSetDevice");
  if ((e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(e, "stream");
  const size_t N = (size_t)n;
  if ((e = cudaMalloc(&c->pos, sizeof(md_double4) * N)) != cudaSuccess) return bail(e, "pos");
  double** vecs[] = {&c->vel, &c->acc, &c->b, &c->c, &c->f3, &c->f3_tmp};
  for (double** p : vecs)
    if ((e = cudaMalloc(p, sizeof(double) * 3 * N)) != cudaSuccess) return bail(e, "state");
  if ((e = cudaMalloc(&c->posf, sizeof(float4) * N)) != cudaSuccess) return bail(e, "posf");
  if (c->cluster) {
    if ((e = cudaMalloc(&c->io, sizeof(double) * 4 * N)) != cudaSuccess) return bail(e, "io");
    if ((e = cudaMalloc(&c->pos_alt, sizeof(md_double4) * N)) != cudaSuccess)
      return bail(e, "pos");
    if ((e = cudaMalloc(&c->posf_alt, sizeof(float4) * N)) != cudaSuccess)
      return bail(e, "posf");
  }
  if ((e = cudaMalloc(&c->status, sizeof(int) * 4)) != cudaSuccess) return bail(e, "flags");
  c->wall_flag = c->status + 1;
  c->missing = c->status + 2;
  if ((e = cudaMemset(c->status, 0, sizeof(int) * 4)) != cudaSuccess) return bail(e, "flags");
  if ((e = cudaMalloc(&c->sc.dpart, sizeof(double) * (8 * 1024 + 64))) != cudaSuccess)
    return bail(e, "scratch");
  if ((e = cudaMalloc(&c->sc.umax, sizeof(unsigned long long) * 4)) != cudaSuccess)
    return bail(e, "scratch");
  if ((e = cudaMalloc(&c->sc.counts, sizeof(int) * 8)) != cudaSuccess) return bail(e, "scratch");
  if ((e = cudaMalloc(&c->dsc, sizeof(double) * 40)) != cudaSuccess) return bail(e, "scratch");
  cudaMemsetAsync(c->dsc, 0, sizeof(double) * 40, c->st);
  *out = c;
  return MD_OK;
}

void md_destroy(md_ctx* c) {
  if (!c) return;
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->io_st) {
    cudaStreamSynchronize(c->io_st);
    cudaStreamDestroy(c->io_st);
  }
  for (float* h : c->anim_blocks) cudaFreeHost(h);
  for (int k = 0; k < 2; k++) {
    if (c->anim_ready[k]) cudaEventDestroy(c->anim_ready[k]);
    if (c->anim_done[k]) cudaEventDestroy(c->anim_done[k]);
  }
  if (c->anim_dev) cudaFree(c->anim_dev);
  list_free(c->lj);
  list_free(c->mb);
  cluster_free(c->cl);
  for (cudaGraphExec_t x : c->gexec)
    if (x) cudaGraphExecDestroy(x);
  void* ptrs[] = {c->sur_flags, c->seq_buf, c->inv, c->sur_fx, c->sur_fs, c->rep_ranges, c->rep_buf, c->io, c->pos_alt, c->posf_alt, c->pos, c->vel, c->acc, c->b, c->c, c->f3, c->f3_tmp, c->posf, c->mb_sl,
                  c->mb_slen, c->xsi, c->xsj, c->status, c->epart, c->dsc, c->rec,
                  c->sc.dpart, c->sc.umax, c->sc.counts, c->sc.block_sums};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& p : c->pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

md_status md_upload(md_ctx* c, const double* pos4, const double* vel3) {
  return md_upload_state(c, pos4, vel3, nullptr, nullptr, nullptr);
}

// host -> device array of `width` doubles per atom, in the caller's numbering
// the device address of a caller buffer the GPU reaches directly (pinned
// host memory, e.g. from md_host_alloc), else NULL
const void* device_view(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

md_status ensure_inv(md_ctx* c) {
  if (!c->inv) CK(cudaMalloc(&c->inv, sizeof(int) * (size_t)c->n), "inverse order");
  if (c->inv_version != c->cl.version) {
    launch_invert(c->cl.orig, c->inv, c->n, c->st);
    c->inv_version = c->cl.version;
  }
  return MD_OK;
}

// Caller -> device.  In cell order, a pinned caller array is read by the
// device in place (whole lines over the host link, no staging copy);
// other memory goes through the staging buffer.  The caller synchronises.
md_status put_array(md_ctx* c, double* dst, const double* src, int width) {
  const size_t B = sizeof(double) * (size_t)width * (size_t)c->n;
  if (!c->permuted()) {
    CK(cudaMemcpyAsync(dst, src, B, cudaMemcpyHostToDevice, c->st), "upload");
    return MD_OK;
  }
  if (const double* hv = (const double*)device_view(src)) {
    md_status s = ensure_inv(c);
    if (s != MD_OK) return s;
    launch_gather_host(hv, dst, c->inv, c->n, width, c->st);
    return MD_OK;
  }
  CK(cudaMemcpyAsync(c->io, src, B, cudaMemcpyHostToDevice, c->st), "upload");
  launch_permute_in(c->io, dst, c->cl.orig, c->n, width, c->st);
  // io is reused by the next transfer: complete this one first
  CK(cudaStreamSynchronize(c->st), "upload");
  return MD_OK;
}

md_status get_array(md_ctx* c, double* dst, const double* src, int width) {
  const size_t B = sizeof(double) * (size_t)width * (size_t)c->n;
  if (!c->permuted()) {
    CK(cudaMemcpyAsync(dst, src, B, cudaMemcpyDeviceToHost, c->st), "download");
    return MD_OK;
  }
  if (double* hv = (double*)device_view(dst)) {
    md_status s = ensure_inv(c);
    if (s != MD_OK) return s;
    launch_scatter_host(src, hv, c->inv, c->n, width, c->st);
    return MD_OK;
  }
  launch_unpermute(src, c->io, c->cl.orig, c->n, width, c->st);
  CK(cudaMemcpyAsync(dst, c->io, B, cudaMemcpyDeviceToHost, c->st), "download");
  CK(cudaStreamSynchronize(c->st), "download");
  return MD_OK;
}

md_status md_upload_state(md_ctx* c, const double* pos4, const double* vel3, const double* a3,
                          const double* b3, const double* c3) {
  if (!c) return MD_BAD_ARGUMENT;
  md_status s = MD_OK;
  int* other = c->status + 3;  // some atom is not of the NG species
  if (pos4) {
    if ((s = put_array(c, (double*)c->pos, pos4, 4)) != MD_OK) return s;
    CK(cudaMemsetAsync(other, 0, sizeof(int), c->st), "upload");
    launch_species_check(c->pos, c->n, other, c->st);
  }
  if (vel3 && (s = put_array(c, c->vel, vel3, 3)) != MD_OK) return s;
  if (a3 && (s = put_array(c, c->acc, a3, 3)) != MD_OK) return s;
  if (b3 && (s = put_array(c, c->b, b3, 3)) != MD_OK) return s;
  if (c3 && (s = put_array(c, c->c, c3, 3)) != MD_OK) return s;
  if (c->mixed() && pos4) launch_posf(c->pos, c->posf, c->n, c->st);
  int flag = 0;
  if (pos4) CK(cudaMemcpyAsync(&flag, other, sizeof(int), cudaMemcpyDeviceToHost, c->st), "upload");
  CK(cudaStreamSynchronize(c->st), "upload");
  if (pos4) c->all_ng = flag == 0;
  return MD_OK;
}

md_status md_download(md_ctx* c, double* pos4, double* vel3) {
  if (!c) return MD_BAD_ARGUMENT;
  md_status s = MD_OK;
  if (pos4 && (s = get_array(c, pos4, (const double*)c->pos, 4)) != MD_OK) return s;
  if (vel3 && (s = get_array(c, vel3, c->vel, 3)) != MD_OK) return s;
  CK(cudaStreamSynchronize(c->st), "download");
  return MD_OK;
}

md_status md_download_state(md_ctx* c, double* a3, double* b3, double* c3, double* f3) {
  if (!c) return MD_BAD_ARGUMENT;
  md_status s = MD_OK;
  if (a3 && (s = get_array(c, a3, c->acc, 3)) != MD_OK) return s;
  if (b3 && (s = get_array(c, b3, c->b, 3)) != MD_OK) return s;
  if (c3 && (s = get_array(c, c3, c->c, 3)) != MD_OK) return s;
  if (f3 && (s = get_array(c, f3, c->f3, 3)) != MD_OK) return s;
  CK(cudaStreamSynchronize(c->st), "download");
  return MD_OK;
}

md_status md_begin(md_ctx* c, float vxcm) {
  if (!c) return MD_BAD_ARGUMENT;
  const size_t B = sizeof(double) * 3 * (size_t)c->n;
  CK(cudaMemsetAsync(c->acc, 0, B, c->st), "begin");
  CK(cudaMemsetAsync(c->b, 0, B, c->st), "begin");
  CK(cudaMemsetAsync(c->c, 0, B, c->st), "begin");
  CK(cudaMemsetAsync(c->status, 0, sizeof(int) * 4, c->st), "begin");
  k_begin<<<(c->n + 255) / 256, 256, 0, c->st>>>(c->pos, c->vel, c->n, c->box_size / 2,
                                                  c->walls(), (double)vxcm);
  c->stats = md_stats{};
  c->stats.launches = 1;
  c->t = 0;
  c->lj_next = c->mb_next = 0;
  c->printout = c->cfg.output_timesteps;
  c->nrec = 0;
  c->begun = true;
  c->predicted = false;
  md_status s = rebuild(c, 0);
  if (s != MD_OK) return s;
  if (c->cfg.output_timesteps > 0) {
    s = push_record(c, 0);
    if (s != MD_OK) return s;
  }
  // the frames of a run start with the state before its first step
  // (cpu/cpumd/Host.cpp:126-127; flushVectors clears them per run)
  c->anim_frames = 0;
  if (c->anim_every >= 0) {
    s = capture_frame(c);
    if (s != MD_OK) return s;
    c->anim_next = c->anim_every;
  }
  forces(c, c->f3);
  launch_accel(c->pos, c->acc, c->f3, c->n, c->sp, c->st);
  c->stats.launches++;
  return check_status(c);
}

md_status md_step(md_ctx* c, int nsteps) {
  if (!c || nsteps < 0) return MD_BAD_ARGUMENT;
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  {
    Timed whole(c, 5);
    for (int s = 0; s < nsteps;) {
      md_status r;
      if (window_ok(c, s, nsteps)) {
        r = run_window(c);
        s += kGraphSteps;
      } else {
        r = step_once(c, s == nsteps - 1);
        s++;
      }
      if (r != MD_OK) return r;
    }
  }
  md_status r = check_status(c);
  if (c->timing) resolve_timing(c);
  return r;
}

int md_record_count(const md_ctx* c) { return c ? c->nrec : 0; }

md_status md_get_records(md_ctx* c, md_thermo* out, int max_records) {
  if (!c || (!out && max_records > 0)) return MD_BAD_ARGUMENT;
  int n = c->nrec < max_records ? c->nrec : max_records;
  static_assert(sizeof(md_thermo) == 16 * sizeof(double), "md_thermo layout");
  if (n > 0)
    CK(cudaMemcpyAsync(out, c->rec, sizeof(md_thermo) * (size_t)n, cudaMemcpyDeviceToHost, c->st), "records");
  CK(cudaStreamSynchronize(c->st), "records");
  return MD_OK;
}

md_status md_thermo_now(md_ctx* c, md_thermo* out) {
  if (!c || !out) return MD_BAD_ARGUMENT;
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  double* tmp = c->dsc + 16;
  md_status s = make_record(c, c->t, tmp);
  if (s != MD_OK) return s;
  CK(cudaMemcpyAsync(out, tmp, sizeof(md_thermo), cudaMemcpyDeviceToHost, c->st), "thermo");
  CK(cudaStreamSynchronize(c->st), "thermo");
  return MD_OK;
}

md_status md_reference_potential(md_ctx* c, double* vib_lj, double* vib_mb) {
  if (!c) return MD_BAD_ARGUMENT;
  md_status s = ensure_epart(c, 2LL * c->n);
  if (s != MD_OK) return s;
  launch_ref_potential(c->pos, c->n, c->sp, c->epart, c->dsc + 14, c->st);
  double r[2];
  CK(cudaMemcpyAsync(r, c->dsc + 14, sizeof(r), cudaMemcpyDeviceToHost, c->st), "potential");
  CK(cudaStreamSynchronize(c->st), "potential");
  if (vib_lj) *vib_lj = r[0];
  if (vib_mb) *vib_mb = r[1];
  return MD_OK;
}

md_status md_compute_forces(md_ctx* c, double* f3, double* energy5) {
  if (!c) return MD_BAD_ARGUMENT;
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  double e[16];
  md_status s = make_record(c, c->t, c->dsc + 16);
  if (s != MD_OK) return s;
  CK(cudaMemcpyAsync(e, c->dsc, sizeof(double) * 16, cudaMemcpyDeviceToHost, c->st), "forces");
  // forces of the same evaluation as Host.cpp:132-135 (f3_tmp holds LJ then
  // bond order written by the energy kernels without accumulation; redo it)
  forces(c, c->f3_tmp);
  if (f3) {
    md_status gs = get_array(c, f3, c->f3_tmp, 3);
    if (gs != MD_OK) return gs;
  }
  CK(cudaStreamSynchronize(c->st), "forces");
  if (energy5) {
    energy5[0] = e[8];
    energy5[1] = e[9];
    energy5[2] = e[10];
    energy5[3] = e[11];
    energy5[4] = e[12] + e[13];
  }
  return check_status(c);
}

md_status md_neighbor_list(md_ctx* c, int which, int* rows, signed char* images,
                           long long capacity, int* nlistsize, int* nlargest) {
  if (!c || (which != 0 && which != 1)) return MD_BAD_ARGUMENT;
  if (which == 0 && c->cluster) {
    if (!c->cl.built) return fail(c, MD_BAD_ARGUMENT, "list not built (call md_begin)");
    if (c->batch) return fail(c, MD_BAD_ARGUMENT, "reference rows of a batch: not available");
    long long nls = 27LL * c->cl.maxcell;
    if (nls > c->n - 1) nls = c->n - 1;
    if (nls < 0) nls = 0;
    int* d_rows = nullptr;
    signed char* d_img = nullptr;
    int* d_nl = c->sc.counts;
    CK(cudaMemsetAsync(d_nl, 0, sizeof(int), c->st), "list rows");
    const long long need = nls * c->n;
    if (rows && capacity < need) return fail(c, MD_LIST_OVERFLOW, "rows buffer too small");
    if (rows && need > 0) {
      CK(cudaMalloc(&d_rows, sizeof(int) * (size_t)need), "list rows");
      if (images && cudaMalloc(&d_img, (size_t)need) != cudaSuccess) {
        cudaFree(d_rows);
        return fail(c, MD_OUT_OF_MEMORY, "list images");
      }
    }
    cluster_reference_rows(c->cl, c->pos, (int)nls, d_rows, d_img, d_nl, c->st);
    int h_nl = 0;
    cudaError_t e = cudaMemcpyAsync(&h_nl, d_nl, sizeof(int), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess && d_rows)
      e = cudaMemcpyAsync(rows, d_rows, sizeof(int) * (size_t)need, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess && d_img)
      e = cudaMemcpyAsync(images, d_img, (size_t)need, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (d_rows) cudaFree(d_rows);
    if (d_img) cudaFree(d_img);
    if (e != cudaSuccess) return cuda_fail(c, e, "list rows");
    if (nlistsize) *nlistsize = (int)nls;
    if (nlargest) *nlargest = h_nl;
    return MD_OK;
  }
  NeighborList& nl = which == 0 ? c->lj : c->mb;
  if (!nl.cell3) return fail(c, MD_BAD_ARGUMENT, "list not built (call md_begin)");
  if (nlistsize) *nlistsize = nl.nlistsize;
  if (nlargest) *nlargest = nl.nlargest;
  const long long need = (long long)nl.nlistsize * nl.n;
  if (!rows) return MD_OK;
  if (capacity < need) return fail(c, MD_LIST_OVERFLOW, "rows buffer too small");
  if (need == 0) return MD_OK;
  int* d_rows = nullptr;
  signed char* d_img = nullptr;
  CK(cudaMalloc(&d_rows, sizeof(int) * (size_t)need), "list rows");
  if (images && cudaMalloc(&d_img, (size_t)need) != cudaSuccess) {
    cudaFree(d_rows);
    return fail(c, MD_OUT_OF_MEMORY, "list images");
  }
  list_reference_rows(nl, c->pos, d_rows, d_img, c->st);
  cudaError_t e = cudaMemcpyAsync(rows, d_rows, sizeof(int) * (size_t)need, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess && images)
    e = cudaMemcpyAsync(images, d_img, (size_t)need, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaFree(d_rows);
  if (d_img) cudaFree(d_img);
  if (e != cudaSuccess) return cuda_fail(c, e, "list rows");
  return MD_OK;
}

md_status md_get_stats(const md_ctx* c, md_stats* out) {
  if (!c || !out) return MD_BAD_ARGUMENT;
  *out = c->stats;
  int* skin = c->cluster ? c->cl.skin : c->lj.skin;
  if (skin) {
    // skin refreshes since the last list build are still on the device
    int sk[5] = {0, 0, 0, 0, 0};
    const size_t words = c->cluster ? 5 : 4;  // the row-list flags hold 4 ints
    if (cudaStreamSynchronize(c->st) != cudaSuccess ||
        cudaMemcpy(sk, skin, sizeof(int) * words, cudaMemcpyDeviceToHost) != cudaSuccess)
      return MD_CUDA_ERROR;
    out->list_trips += c->cluster ? sk[4] : sk[3];
  }
  return MD_OK;
}

md_status md_autotune(md_ctx* c, int evals, md_tune_result* out) {
  if (!c || evals < 1) return MD_BAD_ARGUMENT;
  if (out) memset(out, 0, sizeof(*out));
  if (!c->cluster) return MD_OK;  // only the cluster kernel has tiles to pick
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  const bool fixed_threads = c->cfg.cluster_threads > 0;
  std::vector<int> threads = fixed_threads ? std::vector<int>{c->cl.block}
                                           : std::vector<int>{64, 96, 128, 160, 192};
  // Stage caps: two fixed ones and the largest at which the fused kernel
  // keeps the blocks per SM its registers allow.  An unbounded stage (one
  // block fewer per SM on 1M argon atoms) timed 5% faster here, right after
  // a build, and 3% slower in the step loop (0.2105 against 0.2050 ms).
  auto caps_for = [&](int t, int ld) {
    if (c->cfg.cluster_stage_cap > 0) return std::vector<int>{c->cfg.cluster_stage_cap};
    std::vector<int> v{1152, 1536};
    const int occ = cluster_occupancy_cap(t, ld, c->all_ng != 0);
    if (occ != 1152 && occ != 1536) v.push_back(occ);
    return v;
  };
  const std::vector<int> loads = c->cfg.cluster_row_loads > 0
                                     ? std::vector<int>{c->cfg.cluster_row_loads}
                                     : std::vector<int>{1, 2, 3, 4};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "autotune");
  CK(cudaEventCreate(&e1), "autotune");
  double best = 1e300;
  int best_t = c->cl.block, best_c = c->cl.stage_cap, best_l = c->cl.row_loads, tried = 0;
  std::vector<ClusterReplica> reps = cluster_reps(c);
  double** v3[5] = {&c->vel, &c->acc, &c->b, &c->c, &c->f3};
  // Where steps fuse the Gear update into the force kernel, candidates are
  // timed as that kernel, on a scratch copy of the Gear state and scratch
  // skin flags (the timing leaves the trajectory untouched).
  const bool fused = c->mixed() && !c->walls();
  const size_t n3 = 3 * (size_t)c->n;
  double* gs = nullptr;
  int* skin_s = nullptr;
  if (fused) {
    CK(cudaMalloc(&gs, sizeof(double) * 4 * n3), "autotune scratch");
    if (cudaMalloc(&skin_s, sizeof(int) * 8) != cudaSuccess) {
      cudaFree(gs);
      return cuda_fail(c, cudaErrorMemoryAllocation, "autotune scratch");
    }
  }
  ClusterGearArgs cg;
  auto launch = [&]() {
    ClusterForceArgs a = cl_args(c, c->f3_tmp, nullptr);
    if (fused) {
      a.gear = &cg;
      a.skin = skin_s;
    }
    launch_lj_cluster(a, false, c->st);
  };
  auto build = [&](int t, int cap, int ld) -> md_status {
    c->cl.block = t;
    c->cl.stage_cap = cap;
    c->cl.row_loads = ld;
    std::string e;
    int r = cluster_build(c->cl, reps, c->cfg.lj_rs, sqrt((double)c->lj_rcutsq), &c->pos, v3,
                          c->posf, c->sc, c->status, c->st, e);
    if (r == -1) return fail(c, MD_BAD_CONFIG, e);
    if (r != 0) return cuda_fail(c, (cudaError_t)r, "autotune build");
    return MD_OK;
  };
  md_status s = MD_OK;
  std::vector<int3> cand;
  for (int ld : loads)
    for (int t : threads)
      for (int cap : caps_for(t, ld)) cand.push_back(make_int3(ld, t, cap));
  for (const int3& k3 : cand) {
      const int ld = k3.x, t = k3.y, cap = k3.z;
      if ((s = build(t, cap, ld)) != MD_OK) break;
      if (fused) {
        // the build put the state in cell order: copy it after each build
        double* src[4] = {c->vel, c->acc, c->b, c->c};
        for (int k = 0; k < 4; k++)
          cudaMemcpyAsync(gs + k * n3, src[k], sizeof(double) * n3, cudaMemcpyDeviceToDevice,
                          c->st);
        cudaMemsetAsync(skin_s, 0, sizeof(int) * 8, c->st);
        GearArgs g = gear_args(c, c->t + 1);
        cg.pos_next = c->pos_alt;
        cg.posf_next = c->posf_alt;
        cg.vel = gs;
        cg.acc = gs + n3;
        cg.b = gs + 2 * n3;
        cg.c = gs + 3 * n3;
        cg.k = c->gear;
        for (int k = 0; k < 3; k++) cg.inv_mass[k] = g.inv_mass[k];
        cg.trip2 = g.trip2;
      }
      launch();  // warm
      cudaEventRecord(e0, c->st);
      for (int k = 0; k < evals; k++) launch();
      cudaEventRecord(e1, c->st);
      cudaError_t ce = cudaEventSynchronize(e1);
      float ms = 0;
      if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
      if (ce != cudaSuccess) {
        s = cuda_fail(c, ce, "autotune");
        break;
      }
      tried++;
      if (ms < best) {
        best = ms;
        best_t = t;
        best_c = cap;
        best_l = ld;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (fused) {
    cudaStreamSynchronize(c->st);
    cudaFree(gs);
    cudaFree(skin_s);
  }
  if (s != MD_OK) return s;
  if ((s = build(best_t, best_c, best_l)) != MD_OK) return s;
  c->stats.cluster_segments = c->cl.nseg;
  c->stats.cluster_max_staged = c->cl.max_staged;
  if (out) {
    out->threads = best_t;
    out->stage_cap = best_c;
    out->row_loads = best_l;
    out->candidates = tried;
    out->best_ms = best / evals;
  }
  return check_status(c);
}

md_status md_set_animation(md_ctx* c, int every, int frames_hint) {
  if (!c) return MD_BAD_ARGUMENT;
  if (every < 0) {
    c->anim_every = -1;
    return MD_OK;
  }
  const size_t fb = sizeof(float) * 7 * (size_t)c->n;
  if (!c->anim_dev) {
    CK(cudaMalloc(&c->anim_dev, 2 * fb), "animation");
    CK(cudaStreamCreateWithFlags(&c->io_st, cudaStreamNonBlocking), "animation");
    for (int k = 0; k < 2; k++) {
      CK(cudaEventCreateWithFlags(&c->anim_ready[k], cudaEventDisableTiming), "animation");
      CK(cudaEventCreateWithFlags(&c->anim_done[k], cudaEventDisableTiming), "animation");
    }
  }
  if (c->anim_blocks.empty()) {
    // the first pinned block holds frames_hint frames (at most 1 GB), so
    // runs within the hint never allocate while stepping
    const size_t cap = std::max<size_t>(1, ((size_t)1 << 30) / fb);
    c->anim_per_block = (int)std::max<size_t>(
        1, std::min<size_t>(frames_hint > 0 ? (size_t)frames_hint : 16, cap));
    float* h = nullptr;
    CK(cudaHostAlloc((void**)&h, fb * (size_t)c->anim_per_block, cudaHostAllocDefault),
       "animation frames");
    c->anim_blocks.push_back(h);
  }
  c->anim_every = every;
  return MD_OK;
}

int md_animation_count(const md_ctx* c) { return c ? c->anim_frames : 0; }

md_status md_choose_velocities(md_ctx* c, double temperature, unsigned long long seed) {
  if (!c || !(temperature >= 0)) return MD_BAD_ARGUMENT;
  md_status s = choose_velocities(c, temperature, seed);
  if (s != MD_OK) return s;
  return check_status(c);
}

md_status md_set_equilibration(md_ctx* c, double temperature, unsigned long long seed,
                               int every) {
  if (!c || !(temperature >= 0)) return MD_BAD_ARGUMENT;
  c->equi_every = every > 0 ? every : 0;
  c->equi_temp = temperature;
  c->equi_seed = seed;
  c->equi_draws = 0;
  return MD_OK;
}

md_status md_get_animation_frame(md_ctx* c, int k, float* pos4, float* vel3) {
  if (!c || k < 0 || k >= c->anim_frames || (!pos4 && !vel3)) return MD_BAD_ARGUMENT;
  CK(cudaStreamSynchronize(c->io_st), "animation");
  const size_t n = (size_t)c->n;
  const float* f = c->anim_blocks[k / c->anim_per_block] + (size_t)(k % c->anim_per_block) * 7 * n;
  if (pos4) memcpy(pos4, f, sizeof(float) * 4 * n);
  if (vel3) memcpy(vel3, f + 4 * n, sizeof(float) * 3 * n);
  return MD_OK;
}

// common/Results.cpp:51-86: header (atoms, animation timesteps, frames), every
// frame's positions, then every frame's velocities
md_status md_write_animation(md_ctx* c, const char* anim_file, float vxcm) {
  if (!c || !anim_file) return MD_BAD_ARGUMENT;
  if (c->io_st) CK(cudaStreamSynchronize(c->io_st), "animation");
  std::string name = std::string(anim_file) + "(vxcm-";
  {
    char buf[64];
    // the reference streams the float with the default ostream format
    std::snprintf(buf, sizeof(buf), "%g", (double)vxcm);
    name += buf;
  }
  name += ").anm";
  FILE* fp = std::fopen(name.c_str(), "wb");
  if (!fp) return fail(c, MD_BAD_ARGUMENT, "cannot open " + name);
  const int nop = c->n, every = c->anim_every, count = c->anim_frames;
  bool ok = std::fwrite(&nop, sizeof(int), 1, fp) == 1 &&
            std::fwrite(&every, sizeof(int), 1, fp) == 1 &&
            std::fwrite(&count, sizeof(int), 1, fp) == 1;
  const size_t n = (size_t)c->n;
  for (int part = 0; part < 2 && ok; part++)
    for (int k = 0; k < count && ok; k++) {
      const float* f =
          c->anim_blocks[k / c->anim_per_block] + (size_t)(k % c->anim_per_block) * 7 * n;
      const size_t m = part == 0 ? 4 * n : 3 * n;
      ok = std::fwrite(part == 0 ? f : f + 4 * n, sizeof(float), m, fp) == m;
    }
  ok = std::fclose(fp) == 0 && ok;
  return ok ? MD_OK : fail(c, MD_BAD_ARGUMENT, "error writing " + name);
}

md_status md_tail_pairs(md_ctx* c, int* pairs, int capacity, int* count) {
  if (!c || !count || capacity < 0 || (capacity > 0 && !pairs)) return MD_BAD_ARGUMENT;
  *count = 0;
  // many-body atoms are the first n_mb in the caller's numbering; the cell
  // order of the cluster path only exists without them
  if (c->cfg.n_mb < 2 || c->permuted()) return MD_OK;
  int r = tail_pairs(c->pos, c->cfg.n_mb, pairs, capacity, count, c->st);
  if (r) return cuda_fail(c, (cudaError_t)r, "tail pairs");
  return MD_OK;
}

md_status md_set_graphs(md_ctx* c, int on) {
  if (!c) return MD_BAD_ARGUMENT;
  c->graphs = on && c->cluster;
  return MD_OK;
}

md_status md_set_wait_limit(md_ctx* c, int tries) {
  if (!c || tries < 0) return MD_BAD_ARGUMENT;
  c->wait_limit = tries;
  return MD_OK;
}

md_status md_batch_create(const md_config* cfg, int nrep, const int* natoms, const double* boxes,
                          md_ctx** out) {
  if (!cfg || !out || !natoms || !boxes || nrep < 1) return MD_BAD_ARGUMENT;
  *out = nullptr;
  if (cfg->precision != MD_PREC_MIXED || !cfg->use_lj || (cfg->use_mb && cfg->n_mb > 0) ||
      cfg->output_timesteps > 0)
    return MD_BAD_CONFIG;
  long long total = 0;
  double bmin = 1e300;
  for (int k = 0; k < nrep; k++) {
    if (natoms[k] < 1 || !(boxes[k] > 2.0 * (double)cfg->lj_rs)) return MD_BAD_CONFIG;
    total += natoms[k];
    bmin = fmin(bmin, boxes[k]);
  }
  if (total > kMaxAtoms) return MD_BAD_CONFIG;
  md_config c1 = *cfg;
  c1.n_lj = (int)total;
  c1.n_mb = 0;
  c1.use_mb = 0;
  c1.periodic = 1;
  c1.box = bmin;
  c1.lj_kernel = MD_LJ_CLUSTER;
  md_ctx* c = nullptr;
  md_status s = md_create(&c1, &c);
  if (s != MD_OK) return s;
  c->batch = true;
  c->reps_in.assign(nrep, ClusterReplica{});
  std::vector<int> ranges(2 * (size_t)nrep);
  int a0 = 0;
  for (int k = 0; k < nrep; k++) {
    memset(&c->reps_in[k], 0, sizeof(ClusterReplica));
    c->reps_in[k].n = natoms[k];
    c->reps_in[k].L = boxes[k];
    ranges[2 * k] = a0;
    ranges[2 * k + 1] = natoms[k];
    a0 += natoms[k];
  }
  cudaError_t e;
  if ((e = cudaMalloc(&c->rep_ranges, sizeof(int) * ranges.size())) != cudaSuccess ||
      (e = cudaMalloc(&c->rep_buf, sizeof(double) * 19 * (size_t)nrep)) != cudaSuccess ||
      (e = cudaMemcpy(c->rep_ranges, ranges.data(), sizeof(int) * ranges.size(),
                      cudaMemcpyHostToDevice)) != cudaSuccess) {
    md_destroy(c);
    return e == cudaErrorMemoryAllocation ? MD_OUT_OF_MEMORY : MD_CUDA_ERROR;
  }
  *out = c;
  return MD_OK;
}

int md_batch_size(const md_ctx* c) { return c && c->batch ? (int)c->reps_in.size() : 0; }

md_status md_batch_records(md_ctx* c, md_thermo* out, int max_records) {
  if (!c || !out) return MD_BAD_ARGUMENT;
  if (!c->batch) return fail(c, MD_BAD_ARGUMENT, "not a batch context");
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  const int nrep = (int)c->reps_in.size();
  const int B = cluster_blocks(c->cl);
  md_status s = ensure_epart(c, 3LL * (B > 0 ? B : 1));
  if (s != MD_OK) return s;
  double* e3 = c->rep_buf;
  double* rec = c->rep_buf + 3 * (size_t)nrep;
  launch_lj_cluster(cl_args(c, c->f3_tmp, c->epart), true, c->st);
  launch_rep_energy(c->cl, c->epart, e3, c->st);
  launch_rep_records(c->pos, c->vel, c->rep_ranges, nrep, c->sp, e3,
                     (double)c->t * (double)c->cfg.dt, (double)c->t, rec, c->st);
  c->stats.launches += 3;
  const int n = nrep < max_records ? nrep : max_records;
  if (n > 0)
    CK(cudaMemcpyAsync(out, rec, sizeof(md_thermo) * (size_t)n, cudaMemcpyDeviceToHost, c->st),
       "batch records");
  CK(cudaStreamSynchronize(c->st), "batch records");
  return check_status(c);
}

md_status md_surrogate_create(int device, unsigned long long seed, float cutoff,
                              md_surrogate** out) {
  if (!out || !(cutoff > 0.5f)) return MD_BAD_ARGUMENT;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return MD_NO_DEVICE;
  md_surrogate* s = new md_surrogate();
  s->device = device;
  s->rc = cutoff;
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      sur_init(*s, seed, s->stream) != 0) {
    delete s;
    return MD_CUDA_ERROR;
  }
  *out = s;
  return MD_OK;
}

void md_surrogate_destroy(md_surrogate* s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  delete s;
}

int md_surrogate_param_count(void) { return sur_param_count(); }

md_status md_surrogate_collect(md_surrogate* s, md_ctx* c, int stride, int offset, int* added) {
  if (!s || !c || stride < 1 || offset < 0) return MD_BAD_ARGUMENT;
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  if (!c->cfg.use_mb || c->cfg.n_mb < 1 || !c->mb.cell3)
    return fail(c, MD_BAD_ARGUMENT, "no bond-order atoms");
  if (s->rc > c->cfg.mb_rcut + 1e-6f)
    return fail(c, MD_BAD_ARGUMENT, "descriptor cutoff beyond the bond-order cutoff");
  const int n = c->cfg.n_mb;
  int r = sur_descriptors(*s, c->pos, n, make_walker(c->mb), false, c->status, c->st);
  if (r) return cuda_fail(c, (cudaError_t)r, "surrogate descriptors");
  const int B = mb_blocks(n);
  md_status ms = ensure_epart(c, 3LL * B);
  if (ms != MD_OK) return ms;
  MbArgs a = mb_args(c, c->f3_tmp, 0);
  a.epart1 = c->epart;
  a.epart2 = c->epart + 2LL * B;
  a.eatom = s->eatom;
  launch_mb(a, c->mixed(), true, c->st);
  r = sur_collect(*s, n, s->eatom, stride, offset, c->st, added);
  if (r) return cuda_fail(c, (cudaError_t)r, "surrogate samples");
  // the whole configuration, for force matching (f3_tmp holds the exact
  // bond-order forces: the energy launch overwrites it)
  r = sur_add_config(*s, c->pos, n, c->mb.grid.box, c->f3_tmp, s->eatom, c->st);
  if (r) return cuda_fail(c, (cudaError_t)r, "surrogate configuration");
  return check_status(c);
}

md_status md_surrogate_train_forces(md_surrogate* s, int steps, float lr, float w_energy,
                                    float w_force, double* loss_energy, double* loss_force) {
  if (!s || steps < 0 || !(lr > 0.f) || w_energy < 0.f || w_force < 0.f) return MD_BAD_ARGUMENT;
  if (s->cfgs.empty()) return MD_BAD_ARGUMENT;
  s->w_energy = w_energy;
  s->w_force = w_force;
  int r = sur_train_fm(*s, steps, lr, loss_energy, loss_force, s->stream);
  if (r == -1) return MD_BAD_ARGUMENT;
  if (r) return MD_CUDA_ERROR;
  int st = 0;
  cudaMemcpy(&st, s->status_d, sizeof(int), cudaMemcpyDeviceToHost);
  return st & ST_TMA_TIMEOUT ? MD_TIMEOUT : MD_OK;
}

md_status md_surrogate_force_grad(md_surrogate* s, const float* x, const float* v, int n,
                                  float* grad) {
  if (!s || !x || !v || !grad || n < 1) return MD_BAD_ARGUMENT;
  return sur_force_grad(*s, x, v, n, grad, s->stream) ? MD_CUDA_ERROR : MD_OK;
}

md_status md_surrogate_train(md_surrogate* s, int steps, int batch, float lr, double* loss) {
  if (!s || steps < 0 || batch < 1 || !(lr > 0.f)) return MD_BAD_ARGUMENT;
  if (s->ns < 1) return MD_BAD_ARGUMENT;
  int r = sur_train(*s, steps, batch, lr, loss, s->stream);
  if (r == -1) return MD_BAD_ARGUMENT;
  if (r) return MD_CUDA_ERROR;
  int st = 0;
  cudaMemcpy(&st, s->status_d, sizeof(int), cudaMemcpyDeviceToHost);
  return st & ST_TMA_TIMEOUT ? MD_TIMEOUT : MD_OK;
}

md_status md_surrogate_samples(const md_surrogate* s, int* count) {
  if (!s || !count) return MD_BAD_ARGUMENT;
  *count = s->ns;
  return MD_OK;
}

md_status md_surrogate_attach(md_ctx* c, md_surrogate* s, double threshold, int check_every) {
  if (!c || check_every < 1) return MD_BAD_ARGUMENT;
  if (s && (!c->cfg.use_mb || c->cfg.n_mb < 1))
    return fail(c, MD_BAD_ARGUMENT, "no bond-order atoms");
  if (s && !s->normalised) return fail(c, MD_BAD_ARGUMENT, "surrogate not trained");
  if (s && s->rc > c->cfg.mb_rcut + 1e-6f)
    return fail(c, MD_BAD_ARGUMENT, "descriptor cutoff beyond the bond-order cutoff");
  if (s && !c->sur_fx) {
    const size_t B = sizeof(double) * 3 * (size_t)c->cfg.n_mb;
    CK(cudaMalloc(&c->sur_fx, B), "surrogate check buffers");
    CK(cudaMalloc(&c->sur_fs, B), "surrogate check buffers");
    CK(cudaMalloc(&c->sur_flags, sizeof(int) * 2), "surrogate flags");
  }
  if (c->sur_flags) CK(cudaMemsetAsync(c->sur_flags, 0, sizeof(int) * 2, c->st), "surrogate flags");
  c->sur = s;
  c->sur_threshold = threshold;
  c->sur_every = check_every;
  c->sur_last_check = -1;
  c->sur_use = false;
  c->sur_err = c->sur_err_max = -1.0;
  c->sur_steps = c->sur_exact_steps = c->sur_checks = c->sur_rejects = c->sur_declined = 0;
  return MD_OK;
}

md_status md_surrogate_report(const md_ctx* c, md_surrogate_stats* out) {
  if (!c || !out) return MD_BAD_ARGUMENT;
  // steps the network was meant to take but declined on the device
  int d[2] = {0, 0};
  if (c->sur_flags) {
    if (cudaStreamSynchronize(c->st) != cudaSuccess ||
        cudaMemcpy(d, c->sur_flags, sizeof(d), cudaMemcpyDeviceToHost) != cudaSuccess)
      return MD_CUDA_ERROR;
  }
  out->surrogate_steps = c->sur_steps - d[1];
  out->exact_steps = c->sur_exact_steps + d[1];
  out->checks = c->sur_checks;
  out->rejected_checks = c->sur_rejects;
  out->last_error = c->sur_err;
  out->max_error = c->sur_err_max;
  out->declined_steps = c->sur_declined + d[1];
  return MD_OK;
}

md_status md_surrogate_forces(md_surrogate* s, md_ctx* c, double* f3, double* energy) {
  if (!s || !c) return MD_BAD_ARGUMENT;
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  if (!c->cfg.use_mb || c->cfg.n_mb < 1) return fail(c, MD_BAD_ARGUMENT, "no bond-order atoms");
  if (!s->normalised) return fail(c, MD_BAD_ARGUMENT, "surrogate not trained");
  const int n = c->cfg.n_mb;
  double* e_dev = c->dsc + 32;
  int r = sur_forces(*s, c->pos, n, make_walker(c->mb), c->f3_tmp, 0, e_dev, c->status, c->st);
  if (r) return cuda_fail(c, (cudaError_t)r, "surrogate forces");
  if (f3)
    CK(cudaMemcpyAsync(f3, c->f3_tmp, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost,
                       c->st),
       "surrogate forces");
  double e = 0;
  CK(cudaMemcpyAsync(&e, e_dev, sizeof(double), cudaMemcpyDeviceToHost, c->st), "surrogate");
  CK(cudaStreamSynchronize(c->st), "surrogate");
  if (energy) *energy = e;
  return check_status(c);
}

md_status md_surrogate_desc_directional(md_surrogate* s, md_ctx* c, const double* e3,
                                        double* q) {
  if (!s || !c || !e3 || !q) return MD_BAD_ARGUMENT;
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  if (!c->cfg.use_mb || c->cfg.n_mb < 1) return fail(c, MD_BAD_ARGUMENT, "no bond-order atoms");
  const int n = c->cfg.n_mb;
  const RowWalker w = make_walker(c->mb);
  int r = sur_descriptors(*s, c->pos, n, w, false, c->status, c->st);
  if (!r) r = sur_directional(*s, c->pos, n, w.g.box, e3, q, c->st);
  if (r) return cuda_fail(c, (cudaError_t)r, "surrogate directional derivative");
  return check_status(c);
}

md_status md_surrogate_descriptors(md_surrogate* s, md_ctx* c, float* g, int normalised) {
  if (!s || !c || !g) return MD_BAD_ARGUMENT;
  if (!c->begun) return fail(c, MD_BAD_ARGUMENT, "md_begin has not been called");
  if (!c->cfg.use_mb || c->cfg.n_mb < 1) return fail(c, MD_BAD_ARGUMENT, "no bond-order atoms");
  if (normalised && !s->normalised) return fail(c, MD_BAD_ARGUMENT, "surrogate not trained");
  const int n = c->cfg.n_mb;
  int r = sur_descriptors(*s, c->pos, n, make_walker(c->mb), normalised != 0, c->status, c->st);
  if (r) return cuda_fail(c, (cudaError_t)r, "surrogate descriptors");
  CK(cudaMemcpyAsync(g, s->X, sizeof(float) * kSurDesc * (size_t)n, cudaMemcpyDeviceToHost,
                     c->st),
     "descriptors");
  CK(cudaStreamSynchronize(c->st), "descriptors");
  return check_status(c);
}

md_status md_surrogate_params(md_surrogate* s, float* params, int set) {
  if (!s || !params) return MD_BAD_ARGUMENT;
  int r = set ? sur_set_params(*s, params, s->stream) : sur_get_params(*s, params, s->stream);
  return r ? MD_CUDA_ERROR : MD_OK;
}

md_status md_surrogate_normalisation(md_surrogate* s, float* mean32, float* istd32,
                                     double* mu_sigma, int set) {
  if (!s) return MD_BAD_ARGUMENT;
  const size_t B = sizeof(float) * kSurDesc;
  if (set) {
    if (!mean32 || !istd32 || !mu_sigma || !(mu_sigma[1] > 0)) return MD_BAD_ARGUMENT;
    if (cudaMemcpy(s->mean_d, mean32, B, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->istd_d, istd32, B, cudaMemcpyHostToDevice) != cudaSuccess)
      return MD_CUDA_ERROR;
    s->mu = mu_sigma[0];
    s->sigma = mu_sigma[1];
    s->normalised = true;
    return MD_OK;
  }
  if (!s->normalised) return MD_BAD_ARGUMENT;
  if (mean32 && cudaMemcpy(mean32, s->mean_d, B, cudaMemcpyDeviceToHost) != cudaSuccess)
    return MD_CUDA_ERROR;
  if (istd32 && cudaMemcpy(istd32, s->istd_d, B, cudaMemcpyDeviceToHost) != cudaSuccess)
    return MD_CUDA_ERROR;
  if (mu_sigma) {
    mu_sigma[0] = s->mu;
    mu_sigma[1] = s->sigma;
  }
  return MD_OK;
}

md_status md_surrogate_loss_grad(md_surrogate* s, const float* x, const float* t, int n,
                                 float* grad, double* loss) {
  if (!s || !x || !t || !grad || !loss || n < 1) return MD_BAD_ARGUMENT;
  return sur_loss_grad(*s, x, t, n, grad, loss, s->stream) ? MD_CUDA_ERROR : MD_OK;
}

md_status md_surrogate_set_model(md_surrogate* s, int kind, int hidden) {
  if (!s) return MD_BAD_ARGUMENT;
  int r = sur_set_model(*s, kind, hidden, s->stream);
  if (r == -1) return MD_BAD_ARGUMENT;
  return r ? MD_CUDA_ERROR : MD_OK;
}

int md_surrogate_head_param_count(int hidden) {
  return hidden == 32 || hidden == 64 || hidden == 128 ? sur_fh_param_count(hidden) : -1;
}

md_status md_surrogate_head_params(md_surrogate* s, float* params, int count, int set) {
  if (!s || !params) return MD_BAD_ARGUMENT;
  int r = sur_fh_params(*s, params, count, set != 0, s->stream);
  if (r == -1) return MD_BAD_ARGUMENT;
  return r ? MD_CUDA_ERROR : MD_OK;
}

md_status md_surrogate_head_scale(md_surrogate* s, double* scale, int set) {
  if (!s || !scale) return MD_BAD_ARGUMENT;
  if (!set) {
    *scale = s->fh_out;
    return MD_OK;
  }
  if (!(*scale > 0.0) || !std::isfinite(*scale)) return MD_BAD_ARGUMENT;
  s->fh_out = *scale;
  return MD_OK;
}

md_status md_surrogate_range(md_surrogate* s, float* lo32, float* hi32, int set) {
  if (!s || !lo32 || !hi32) return MD_BAD_ARGUMENT;
  if (set)
    for (int f = 0; f < 32; f++)
      if (!(lo32[f] <= hi32[f])) return MD_BAD_ARGUMENT;
  int r = sur_range(*s, lo32, hi32, set != 0, s->stream);
  if (r == -1) return MD_BAD_ARGUMENT;
  return r ? MD_CUDA_ERROR : MD_OK;
}

md_status md_surrogate_head_grad(md_surrogate* s, const float* x, const float* v, int n,
                                 float* grad) {
  if (!s || !x || !v || !grad || n < 1) return MD_BAD_ARGUMENT;
  int r = sur_fh_grad(*s, x, v, n, grad, s->stream);
  if (r == -1) return MD_BAD_ARGUMENT;
  return r ? MD_CUDA_ERROR : MD_OK;
}

md_status md_surrogate_net(md_surrogate* s, const float* x, int n, float* t, float* dtdx) {
  if (!s || !x || !t || !dtdx || n < 1) return MD_BAD_ARGUMENT;
  return sur_net_eval(*s, x, n, t, dtdx, s->stream) ? MD_CUDA_ERROR : MD_OK;
}

md_status md_set_timing(md_ctx* c, int on) {
  if (!c) return MD_BAD_ARGUMENT;
  cudaStreamSynchronize(c->st);
  resolve_timing(c);
  c->timing = on != 0;
  for (int k = 0; k < kKernels; k++) {
    c->kt_ms[k] = 0;
    c->kt_n[k] = 0;
  }
  return MD_OK;
}

md_status md_kernel_time(const md_ctx* cc, int kernel, double* total_ms, long long* launches) {
  md_ctx* c = const_cast<md_ctx*>(cc);
  if (!c || kernel < 0 || kernel >= kKernels) return MD_BAD_ARGUMENT;
  cudaStreamSynchronize(c->st);
  resolve_timing(c);
  if (total_ms) *total_ms = c->kt_ms[kernel];
  if (launches) *launches = c->kt_n[kernel];
  return MD_OK;
}

md_status md_synchronize(md_ctx* c) {
  if (!c) return MD_BAD_ARGUMENT;
  return check_status(c);
}

void* md_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

void md_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

}  // extern "C"
