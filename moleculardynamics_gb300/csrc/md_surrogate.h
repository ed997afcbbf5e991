// Learned surrogate of the bond-order term (host interface shared by the
// surrogate kernels and the step engine).
#pragma once
#include <cuda_bf16.h>

#include <vector>

#include "md_internal.h"

namespace mdgb {

constexpr int kSurDesc = 32;  // 16 radial + 16 angular symmetry functions

// Behler symmetry functions: G2_k = sum_j exp(-eta_r (r - rs_k)^2) fc(r) and
// G4_f = pref_f sum_{j<k} (1 + lam_f cos) ^ zeta_f exp(-eta_f (rj^2 + rk^2))
// fc(rj) fc(rk), fc(r) = (cos(pi r / rc) + 1) / 2 for r < rc.
struct DescParams {
  float rc;
  float eta_r;
  float rs[16];
  float eta_a[16], lam[16], pref[16];
  int zeta[16];
};

// One training configuration: the bond-order atoms of a state with their
// neighbour lists, exact forces and exact per-atom energies (device arrays).
struct SurConfig {
  int n = 0;
  double box = 0.0;
  md_double4* pos = nullptr;
  uint32_t* sl = nullptr;
  int* slen = nullptr;
  double* fx = nullptr;     // exact bond-order forces (3 per atom)
  double* eatom = nullptr;  // exact per-atom energies
  float* G = nullptr;       // raw descriptors (32 per atom)
  float* X = nullptr;       // normalised descriptors (set at training)
  float* T = nullptr;       // normalised energies (set at training)
};

}  // namespace mdgb

struct md_surrogate {
  int device = 0;
  unsigned long long seed = 1;
  float rc = 3.0f;                 // descriptor cutoff (angstrom)
  mdgb::DescParams P{};
  // network parameters (FP32 master), Adam moments, gradients, BF16 copies
  float *P_d = nullptr, *M_d = nullptr, *V_d = nullptr, *G_d = nullptr;
  __nv_bfloat16 *W1 = nullptr, *W1T = nullptr, *W2 = nullptr, *W2T = nullptr;
  int adam_step = 0;
  // input and target normalisation (fixed at the first training)
  float *mean_d = nullptr, *istd_d = nullptr;
  double mu = 0.0, sigma = 1.0;
  bool normalised = false;
  // per-system buffers
  int n_alloc = 0;
  long long n_sl = 0;
  uint32_t* sl = nullptr;
  int* slen = nullptr;
  float *X = nullptr, *t = nullptr, *dtdx = nullptr, *gcoef = nullptr, *F32 = nullptr;
  float4* pos32 = nullptr;         // FP32 positions for the neighbour search
  double* eatom = nullptr;
  // training samples: raw descriptors and exact per-atom energies
  int ns = 0, ns_cap = 0;
  float* SG = nullptr;
  double* SE = nullptr;
  long long nsx = 0;
  float *SX = nullptr, *ST = nullptr;
  // scratch
  double *loss_d = nullptr, *scratch = nullptr;
  int* rows_d = nullptr;
  float *Xg = nullptr, *Tg = nullptr;
  long long nxg = 0;
  int* status_d = nullptr;
  cudaStream_t stream = nullptr;   // stream of the calls that take no context
  // force matching: stored configurations, loss weights, force scale
  std::vector<mdgb::SurConfig> cfgs;
  float w_energy = 1.f, w_force = 1.f;
  double force_var = 0.0;          // mean squared exact force component
  int* iota_d = nullptr;           // 0 .. n-1 (rows of a whole configuration)
  long long n_iota = 0;
  float *V = nullptr, *E3 = nullptr;  // per-atom force sensitivity, residuals
  long long n_fm = 0;
  double last_loss_e = 0.0, last_loss_f = 0.0;
  // model kind: 0 the per-atom energy network (tensor cores), 1 the
  // direct-force head (FP32, 32 -> fh_hidden -> fh_hidden -> 32)
  int kind = 0;
  int fh_hidden = 64, fh_np = 0, fh_step = 0;
  float *FP_d = nullptr, *FM_d = nullptr, *FV_d = nullptr, *FG_d = nullptr, *fh_gs = nullptr;
  float *fh_xT = nullptr, *fh_h1T = nullptr, *fh_h2T = nullptr;
  float *fh_d1T = nullptr, *fh_d2T = nullptr, *fh_d3T = nullptr;
  long long fh_n = 0;
  // force units per unit head output: F_rms over the force RMS that
  // outputs drawn with unit variance per component produce on the first
  // training configuration (0 until measured: F_rms alone)
  double fh_out = 0.0;
  // the descriptor range of the force-matching data (normalised units,
  // widened by range_margin of each span): a guarded force call declines
  // a configuration with any atom outside it
  float *xlo_d = nullptr, *xhi_d = nullptr;  // 32 each
  int* oor_d = nullptr;                      // out-of-range flag of the last guarded call
  bool have_range = false;
  float range_margin = 0.1f;
  ~md_surrogate();
};

namespace mdgb {

using Surrogate = ::md_surrogate;

int sur_init(Surrogate& s, unsigned long long seed, cudaStream_t st);
int sur_set_params(Surrogate& s, const float* P, cudaStream_t st);
int sur_get_params(const Surrogate& s, float* P, cudaStream_t st);
int sur_param_count();
// neighbours within rc, then descriptors of atoms [0, n) into s.X
int sur_directional(Surrogate& s, const md_double4* pos, int n, double box, const double* e3,
                    double* q_host, cudaStream_t st);
int sur_descriptors(Surrogate& s, const md_double4* pos, int n, const RowWalker& w,
                    bool normalised, int* d_status, cudaStream_t st);
// appends atoms offset, offset + stride, ... of the last raw descriptors
// with their exact energies eatom (device) to the training set
int sur_collect(Surrogate& s, int n, const double* eatom, int stride, int offset,
                cudaStream_t st, int* added);
int sur_train(Surrogate& s, int steps, int batch, float lr, double* loss, cudaStream_t st);
// stores the configuration whose descriptors were computed last (s.X, s.sl,
// s.slen) with exact forces fx and energies eatom (device arrays of n atoms)
int sur_add_config(Surrogate& s, const md_double4* pos, int n, double box, const double* fx,
                   const double* eatom, cudaStream_t st);
// force matching over the stored configurations: each Adam step takes one
// configuration, with loss w_energy * mean((t - t*)^2) +
// w_force * mean(|F - F*|^2) / force_var
int sur_train_fm(Surrogate& s, int steps, float lr, double* loss_e, double* loss_f,
                 cudaStream_t st);
// parameter gradient of sum_i v_i . dt/dx(x_i) from the training kernel
int sur_force_grad(Surrogate& s, const float* X, const float* V, int n, float* grad,
                   cudaStream_t st);
int sur_loss_grad(Surrogate& s, const float* X, const float* T, int n, float* grad,
                  double* loss, cudaStream_t st);
int sur_net_eval(Surrogate& s, const float* X, int n, float* t, float* dtdx, cudaStream_t st);
// With a descriptor range known, a configuration with an atom's descriptors
// outside it is declined: declined (host, optional) is then set and no forces
// are computed; or, without a host wait, run_exact (device flag, optional) is
// set to 1 (0 otherwise), f3 is left as it was and declined_count (device,
// optional) counts the declined calls, so that exact kernels gated on
// run_exact take the step.
int sur_forces(Surrogate& s, const md_double4* pos, int n, const RowWalker& w, double* f3,
               int accumulate, double* energy_dev, int* d_status, cudaStream_t st,
               bool* declined = nullptr, int* run_exact = nullptr,
               int* declined_count = nullptr);
// the accepted descriptor range (normalised units): read, or set (and use)
int sur_range(Surrogate& s, float* lo, float* hi, bool set, cudaStream_t st);
// model kind (0 energy network, 1 direct-force head with `hidden` units per
// hidden layer: 32, 64 or 128); the head's weights start from the seed
int sur_set_model(Surrogate& s, int kind, int hidden, cudaStream_t st);
int sur_fh_param_count(int hidden);
int sur_fh_params(Surrogate& s, float* P, int count, bool set, cudaStream_t st);
// parameter gradient of sum_i v_i . w(x_i) of the direct-force head (host
// arrays x, v: n x 32), for the comparison with the CPU restatement
int sur_fh_grad(Surrogate& s, const float* X, const float* V, int n, float* grad,
                cudaStream_t st);
// relative RMS of a against b over n atoms (3 components)
int sur_rel_err(const double* a, const double* b, int n, double* scratch, double* err,
                cudaStream_t st);

}  // namespace mdgb
