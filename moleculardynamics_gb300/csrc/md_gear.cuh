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

// Exact FP32 -> FP64 widening by moving the IEEE-754 fields with integer
// operations (sign; exponent rebiased 127 -> 1023; mantissa shifted left by
// 29), keeping the FP64 pipe, which is narrow on this GPU, for the Gear
// arithmetic.  Subnormal inputs become signed zero; infinities and NaNs keep
// an all-ones exponent.
__device__ __forceinline__ double widen_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint32_t ed = e == 0xFFu ? 0x7FFu : e + 896u;
  const uint32_t hi = (u & 0x80000000u) | (e == 0u ? 0u : (ed << 20) | ((u >> 3) & 0xFFFFFu));
  const uint32_t lo = e == 0u ? 0u : u << 29;
  return __hiloint2double((int)hi, (int)lo);
}

// The conversion instruction, in a function of its own: the compiler cannot
// evaluate a call ahead of its branch, so the common path of narrow_rn issues
// nothing on the FP64 pipe (a conversion there costs as much as an FMA).
static __device__ __noinline__ float narrow_slow(double d) { return __double2float_rn(d); }

// FP64 -> FP32 rounded to nearest, ties to even, by integer operations for
// results in the normal FP32 range; zero, tiny, huge and non-finite values
// take the conversion instruction.
__device__ __forceinline__ float narrow_rn(double d) {
  const uint64_t u = (uint64_t)__double_as_longlong(d);
  const uint32_t hi = (uint32_t)(u >> 32);
  const int e = (int)((hi >> 20) & 0x7FFu) - 896;  // FP32 biased exponent
  if (e <= 0 || e >= 255) return narrow_slow(d);
  const uint32_t mf = (uint32_t)(u >> 29) & 0x7FFFFFu;  // top 23 mantissa bits
  const uint32_t rest = (uint32_t)u & 0x1FFFFFFFu;      // the 29 dropped bits
  const uint32_t up = rest > 0x10000000u || (rest == 0x10000000u && (mf & 1u));
  // a carry out of the mantissa moves into the exponent, as rounding does
  return __uint_as_float((hi & 0x80000000u) | (((uint32_t)e << 23) + mf + up));
}

__device__ __forceinline__ bool gear_finite(const GearAtom& s) {
  return isfinite(s.r[0]) && isfinite(s.r[1]) && isfinite(s.r[2]) && isfinite(s.v[0]) &&
         isfinite(s.v[1]) && isfinite(s.v[2]);
}

}  // namespace mdgb
