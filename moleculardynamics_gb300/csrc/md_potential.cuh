// Pair and bond-order potential primitives, templated on the arithmetic type.
//
// T = double reproduces the reference's FP64 expressions (common/arvdwfc.cpp,
// cpu/common/LennardJones.h); T = float is the precision form's arithmetic.
// Float literals stay float literals so that C++ promotion gives the same
// mixed float/double evaluation as the reference.
#pragma once
#include "md_common.cuh"

namespace mdgb {

// FP64: the library functions (the reference's expressions).  FP32 (the
// precision form, within 1e-4 of FP64 by requirement): the hardware
// approximations, a few ulp each -- exp by ex2.approx, tanh from it as
// 1 - 2 / (e^2x + 1) (absolute error about 1e-7), sqrt as x rsqrt(x) (the
// bond-order distances are never 0), quotients by __fdividef.
__device__ __forceinline__ double md_exp(double x) { return exp(x); }
__device__ __forceinline__ float md_exp(float x) { return __expf(x); }
__device__ __forceinline__ double md_tanh(double x) { return tanh(x); }
__device__ __forceinline__ float md_tanh(float x) {
  return 1.0f - __fdividef(2.0f, __expf(2.0f * x) + 1.0f);
}
__device__ __forceinline__ double md_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float md_sqrt(float x) { return x * rsqrtf(x); }
template <typename T>
__device__ __forceinline__ T fdiv(T a, T b) {
  return a / b;
}
template <>
__device__ __forceinline__ float fdiv<float>(float a, float b) {
  return __fdividef(a, b);
}

// common/Getters.cpp:29-78
template <typename T>
__device__ __forceinline__ T get_re(int ti, int tj) {
  return ti == tj ? (ti == SP_N ? (T)MD_reN : (T)MD_reO) : (T)MD_reNO;
}
template <typename T>
__device__ __forceinline__ T get_de(int ti, int tj) {
  return ti == tj ? (ti == SP_N ? (T)MD_deN : (T)MD_deO) : (T)MD_deNO;
}
template <typename T>
__device__ __forceinline__ T get_beta(int ti, int tj) {
  return ti == tj ? (ti == SP_N ? (T)MD_betaN : (T)MD_betaO) : (T)MD_betaNO;
}
template <typename T>
__device__ __forceinline__ T get_r0v(int ti, int tj) {
  return ti == tj ? (ti == SP_N ? (T)MD_reNvdw : (T)MD_reOvdw) : (T)MD_reNOvdw;
}

// common/arvdwfc.cpp:17-21.  sqrt(2.0f/S) is exactly 1 and sqrt(2S) exactly 2.
template <typename T>
__device__ __forceinline__ void attractive(T& va, T& dva, T rij, T De, T beta, T re) {
  va = MD_S * De / (MD_S - 1.0f) * md_exp(-beta * 1.0f * (rij - re));
  dva = beta * 1.0f * va;
}
// common/arvdwfc.cpp:27-31
template <typename T>
__device__ __forceinline__ void repulsive(T& vr, T& dvr, T rij, T De, T beta, T re) {
  vr = De / (MD_S - 1.0f) * md_exp(-beta * 2.0f * (rij - re)) +
       7.0e-8f * md_exp(-10.0f * beta * (rij - re));
  dvr = beta * 2.0f * vr;
}
// common/arvdwfc.cpp:37-48
template <typename T>
__device__ __forceinline__ void vander_waals(T& vdw, T& dvdw, T rij, T r0v) {
  T alfavm = MD_ALFAV * (rij - r0v);
  T eplus = md_exp(alfavm);
  T gmexp = MD_GM * md_exp(-alfavm);
  T a = eplus + gmexp;
  T b = MD_ALFAV * (eplus - gmexp);
  T db = MD_ALFAVSQ * a;
  T v = 1.0f + 50.0f * MD_GM + MD_GMSQ + 10.0f * (MD_GM - 1.0f) * b;
  dvdw = -1.0e-4f * ((10.0f * (MD_GM - 1.0f) * db * a - 2.0f * b * v) / (a * a * a));
  vdw = 1.0e-4f * v / (a * a);
}
// common/arvdwfc.cpp:54-59
template <typename T>
__device__ __forceinline__ void cutoff(T rij, T& fc, T& dfc) {
  T t = md_tanh(MD_ALFA * (rij - MD_R0));
  dfc = -0.5f * MD_ALFA * (1.0f - t * t);
  fc = 0.5f * (1.0f - t);
}

// Angular function of cpu/common/BondOrderFuncs.h:76-77 and its derivative
// prefactor -C/(D+(H-cos)^2)^2 * 2 (H-cos).
template <typename T>
__device__ __forceinline__ void angular(T costhe, T& g, T& gpre) {
  T hc = MD_H - costhe;
  T q = MD_D + hc * hc;
  g = 1.0f + MD_C / MD_D - fdiv<T>(MD_C, q);
  gpre = -fdiv<T>(MD_C, q * q) * 2.0f * hc;
}

// the same with one reciprocal, for the FP32 forms (the FP64 path keeps the
// reference's two quotients)
template <typename T>
__device__ __forceinline__ void angular1(T costhe, T& g, T& gpre) {
  const T hc = MD_H - costhe;
  const T iq = fdiv<T>(1.0f, MD_D + hc * hc);
  g = 1.0f + MD_C / MD_D - MD_C * iq;
  gpre = -MD_C * iq * iq * 2.0f * hc;
}

// LennardJones.h:65-86: parameters of an NG pair, selected by the other type
__device__ __forceinline__ int lj_select(int ti, int tj) { return ti == SP_NG ? tj : ti; }

// LennardJones.h:12-30 in FP64 with every rounding of the reference
// (no FMA contraction): adds r_ij * f_ij to (fx, fy, fz) and returns f_ij.
// sigsq = sig * sig and con = 24 eps / sigsq depend on the species pair only:
// a caller that evaluates them once with these operations gets the same bits
__device__ __forceinline__ double lj_pair_exact_c(double& fx, double& fy, double& fz,
                                                  double dist, double ijx, double ijy,
                                                  double ijz, double sigsq, double con) {
  double dist2 = xdiv(xmul(dist, dist), sigsq);
  double dist4 = xmul(dist2, dist2);
  double dist8 = xmul(dist4, dist4);
  double dist14 = xmul(xmul(dist2, dist4), dist8);
  double invdist8 = xdiv(1.0, dist8);
  double invdist14 = xdiv(1.0, dist14);
  double s = xsub(xmul(2.0, invdist14), invdist8);
  double fij = xmul(s, con);
  fx = xadd(fx, xmul(ijx, fij));
  fy = xadd(fy, xmul(ijy, fij));
  fz = xadd(fz, xmul(ijz, fij));
  return fij;
}

__device__ __forceinline__ double lj_sigsq(double sig) { return xmul(sig, sig); }
__device__ __forceinline__ double lj_con(double eps, double sigsq) {
  return xdiv(xmul(24.0, eps), sigsq);
}

__device__ __forceinline__ double lj_pair_exact(double& fx, double& fy, double& fz,
                                                double dist, double ijx, double ijy,
                                                double ijz, double sig, double eps) {
  const double sigsq = lj_sigsq(sig);
  return lj_pair_exact_c(fx, fy, fz, dist, ijx, ijy, ijz, sigsq, lj_con(eps, sigsq));
}

}  // namespace mdgb
