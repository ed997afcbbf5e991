// Per-atom Gear 5th-order corrector and predictor of the precision form
// (cpu/common/Device.cpp:17-39 predict, :44-85 correct, without walls):
// FP64 state, products fused into FMAs and F/m taken as F * (1/m).  Shared by
// the stand-alone Gear kernel and the fused force + Gear kernel of the
// cluster path, so both advance the state with the same arithmetic.
#pragma once
#include "md_integrate.h"

namespace mdgb {

struct GearAtom {
  double r[3], v[3], a[3], b[3], c[3];
};

// a_new = F/m; d = a_new - a; r, v, b, c += GEAR_k * c2 / c_k * d; a = a_new
__device__ __forceinline__ void gear_correct_fma(GearAtom& s, const double f[3], double inv_mass,
                                                 const GearCoef& k) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double ai = f[d] * inv_mass;
    const double corr = ai - s.a[d];
    s.r[d] = fma(k.cr, corr, s.r[d]);
    s.v[d] = fma(k.cv, corr, s.v[d]);
    s.a[d] = ai;
    s.b[d] = fma(k.cb, corr, s.b[d]);
    s.c[d] = fma(k.cc, corr, s.c[d]);
  }
}

// Taylor predictor: r += c1 v + c2 a + c3 b + c4 c; v += c1 a + c2 b + c3 c; ...
__device__ __forceinline__ void gear_predict_fma(GearAtom& s, const GearCoef& k) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    s.r[d] = fma(k.c4, s.c[d], fma(k.c3, s.b[d], fma(k.c2, s.a[d], fma(k.c1, s.v[d], s.r[d]))));
    s.v[d] = fma(k.c3, s.c[d], fma(k.c2, s.b[d], fma(k.c1, s.a[d], s.v[d])));
    s.a[d] = fma(k.c2, s.c[d], fma(k.c1, s.b[d], s.a[d]));
    s.b[d] = fma(k.c1, s.c[d], s.b[d]);
  }
}

__device__ __forceinline__ bool gear_finite(const GearAtom& s) {
  return isfinite(s.r[0]) && isfinite(s.r[1]) && isfinite(s.r[2]) && isfinite(s.v[0]) &&
         isfinite(s.v[1]) && isfinite(s.v[2]);
}

}  // namespace mdgb
