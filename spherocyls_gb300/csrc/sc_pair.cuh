// sc_pair.cuh -- segment-segment contact of two spherocylinders (device code).
//
// Two forms of the same geometry (tmarschall/spherocyls
// src/cpp/strain_dynamics.cpp:17-75, calc_force_pair; stress arms from
// src/cpp/spherocyl_box.cpp:425-500, calc_se_force_pair):
//
//  * pair_fp64: every floating-point operation in the reference's order.  It is
//    compiled in a translation unit built with -fmad=false so no fused
//    multiply-add changes the rounding; together with role assignment by particle
//    index (the lower index plays the reference's "p") each pair contribution is
//    the reference's up to the last-ulp difference of the device cos/sin.
//  * pair_fp32: the same closest-point algorithm in FP32 on a displacement that
//    the caller already reduced to the minimum image, with fast reciprocal and
//    reciprocal-square-root; the caller accumulates stress and energy in FP64.
//
// Both take the displacement of P relative to Q in sheared coordinates and apply
// the Lees-Edwards shift dX += gamma*dY themselves.
#pragma once

#include <cuda_runtime.h>

namespace sc {

struct PairF64 {
  double fx, fy, tp, tq;          // force on P (Q gets -f), torques on P and Q
  double e, pxx, pyy, pxy, pyx;   // stress/energy contributions (when requested)
};

// dX, dY: raw coordinate differences P - Q (no minimum image yet).
// Returns true when the spherocylinders overlap.
template <bool SE>
__device__ __forceinline__ bool pair_fp64(double dX, double dY, double nxA, double nyA, double aP,
                                          double nxB, double nyB, double aQ, double sig,
                                          double gamma, double Lx, double Ly, bool virial,
                                          double two_n, PairF64& o) {
  dX += Lx * (double)((dX < -0.5 * Lx) - (dX > 0.5 * Lx));
  dY += Ly * (double)((dY < -0.5 * Ly) - (dY > 0.5 * Ly));
  dX += gamma * dY;

  double a = aP * aP;
  double b = -(nxA * nxB + nyA * nyB);
  double c = aQ * aQ;
  double d = nxA * dX + nyA * dY;
  double e = -nxB * dX - nyB * dY;
  double delta = a * c - b * b;

  double t = fmin(fmax((b * d - a * e) / delta, -1.), 1.);
  double s = -(b * t + d) / a;
  double sarg = fabs(s);
  s = fmin(fmax(s, -1.), 1.);
  if (sarg > 1) t = fmin(fmax(-(b * s + e) / c, -1.), 1.);

  double dDx = dX + s * nxA - t * nxB;
  double dDy = dY + s * nyA - t * nyB;
  double dsq = dDx * dDx + dDy * dDy;
  if (!(dsq < sig * sig)) return false;
  double dij = sqrt(dsq);
  double dvij = (1.0 - dij / sig) / sig;
  double Fx = dDx * dvij / dij;
  double Fy = dDy * dvij / dij;
  o.fx = Fx;
  o.fy = Fy;
  o.tp = s * nxA * Fy - s * nyA * Fx;
  o.tq = t * nyB * Fx - t * nxB * Fy;
  if (SE) {
    double LL = Lx * Ly;
    double CxA = s * nxA - 0.5 * dDx;
    double CyA = s * nyA - 0.5 * dDy;
    double CxB = t * nxB + 0.5 * dDx;
    o.e = dvij * sig * (1.0 - dij / sig) / two_n;
    if (!virial) {
      // the reference's accumulation, slips included: CyB is built from nxB,
      // one Pxy term lands in Pxx, and Pxy misses its B arm.
      double CyB = t * nxB + 0.5 * dDy;
      o.pxx = Fx * CxA / LL - Fx * CxB / LL - Fy * CxB / LL;
      o.pyy = Fy * CyA / LL - Fy * CyB / LL;
      o.pxy = Fy * CxA / LL;
      o.pyx = Fx * CyA / LL - Fx * CyB / LL;
    } else {
      double CyB = t * nyB + 0.5 * dDy;
      o.pxx = Fx * CxA / LL - Fx * CxB / LL;
      o.pyy = Fy * CyA / LL - Fy * CyB / LL;
      o.pxy = Fy * CxA / LL - Fy * CxB / LL;
      o.pyx = Fx * CyA / LL - Fx * CyB / LL;
    }
  }
  return true;
}

struct PairF32 {
  float fx, fy, tp, tq;
  float ov;                      // overlap 1 - d/sigma
  float cxa, cya, cxb, cyb;      // contact arms (virial or reference form)
};

// dX, dY: displacement P - Q already reduced to the minimum image (FP32).
template <bool SE>
__device__ __forceinline__ bool pair_fp32(float dX, float dY, float nxA, float nyA, float aP,
                                          float nxB, float nyB, float aQ, float sig, float gamma,
                                          bool virial, PairF32& o) {
  dX = fmaf(gamma, dY, dX);
  float a = aP * aP;
  float b = -(nxA * nxB + nyA * nyB);
  float c = aQ * aQ;
  float d = nxA * dX + nyA * dY;
  float e = -(nxB * dX + nyB * dY);
  // Unclamped spine parameter of Q.  The reference's (b d - a e)/(a c - b^2) is,
  // by the Binet-Cauchy identity, cross(u_A, D)/cross(u_A, u_B); the cross-product
  // form keeps FP32 accurate for nearly parallel spines, where a c - b^2 cancels.
  // Exactly parallel spines give 0/0 in the reference, which its clamp turns into
  // t = -1; the same value is used here.
  float w = nyA * nxB;
  float uxv = fmaf(nxA, nyB, -w) + fmaf(-nyA, nxB, w);  // cross(u_A, u_B), error-compensated
  float w2 = nyA * dX;
  float uxD = fmaf(nxA, dY, -w2) + fmaf(-nyA, dX, w2);  // cross(u_A, D)
  float t = uxv == 0.f ? -1.f : fminf(fmaxf(__fdividef(uxD, uxv), -1.f), 1.f);
  float s = -__fdividef(b * t + d, a);
  float sarg = fabsf(s);
  s = fminf(fmaxf(s, -1.f), 1.f);
  if (sarg > 1.f) t = fminf(fmaxf(-__fdividef(b * s + e, c), -1.f), 1.f);
  float dDx = dX + s * nxA - t * nxB;
  float dDy = dY + s * nyA - t * nyB;
  float dsq = dDx * dDx + dDy * dDy;
  if (!(dsq < sig * sig)) return false;
  float inv_d = rsqrtf(dsq);
  float inv_sig = __frcp_rn(sig);
  float ov = 1.f - dsq * inv_d * inv_sig;   // 1 - d/sigma
  float f = ov * inv_sig * inv_d;           // (1 - d/sigma)/(sigma d)
  float Fx = dDx * f, Fy = dDy * f;
  o.fx = Fx;
  o.fy = Fy;
  o.tp = s * (nxA * Fy - nyA * Fx);
  o.tq = t * (nyB * Fx - nxB * Fy);
  if (SE) {
    o.ov = ov;
    o.cxa = s * nxA - 0.5f * dDx;
    o.cya = s * nyA - 0.5f * dDy;
    o.cxb = t * nxB + 0.5f * dDx;
    o.cyb = (virial ? t * nyB : t * nxB) + 0.5f * dDy;
  }
  return true;
}

// isolated_rotation, src/cpp/strain_dynamics.cpp:174-177
__device__ __forceinline__ double iso_rot64(double RC, double phi) {
  return 0.5 * (1 - RC * cos(2 * phi));
}

__device__ __forceinline__ int wrap_index(int v, int n) {
  return v < 0 ? v + n : (v >= n ? v - n : v);
}

}  // namespace sc
