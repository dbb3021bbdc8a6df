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

// x / y, or, in the minimiser's form (FAST), x times a reciprocal of y shared by
// several quotients.  The FAST form trades the last bits of the reference's
// rounding for fewer FP64 divisions (GB300's FP64 rate is a small fraction of its
// FP32 rate); the force-evaluation and dynamics paths never use it.
template <bool FAST>
__device__ __forceinline__ double qdiv(double x, double y, double inv_y) {
  return FAST ? x * inv_y : x / y;
}

// Reciprocals of a = |u_A|^2, c = |u_B|^2, delta and sig from one division.
struct Recip64 {
  double a, c, delta, sig;
};
__device__ __forceinline__ Recip64 recip64(double a, double c, double delta, double sig) {
  Recip64 r;
  const double ac = a * c;
  if (delta > 0) {
    const double inv = 1.0 / (ac * delta * sig);
    const double i_ac = delta * sig * inv;
    r.delta = ac * sig * inv;
    r.sig = ac * delta * inv;
    r.a = c * i_ac;
    r.c = a * i_ac;
  } else {
    const double inv = 1.0 / (ac * sig);
    r.delta = 0.0;
    r.sig = ac * inv;
    r.a = c * sig * inv;
    r.c = a * sig * inv;
  }
  return r;
}

// dX, dY: raw coordinate differences P - Q (no minimum image yet).
// Returns true when the spherocylinders overlap.
// FAST with SE (the mixed form's FP64 stress): inv_LL = 1/(Lx Ly) and inv_two_n =
// 1/(2n) from the caller replace the per-term divisions.
template <bool SE, bool FAST = false>
__device__ __forceinline__ bool pair_fp64(double dX, double dY, double nxA, double nyA, double aP,
                                          double nxB, double nyB, double aQ, double sig,
                                          double gamma, double Lx, double Ly, bool virial,
                                          double two_n, PairF64& o, double inv_LL = 0.0,
                                          double inv_two_n = 0.0) {
  dX += Lx * (double)((dX < -0.5 * Lx) - (dX > 0.5 * Lx));
  dY += Ly * (double)((dY < -0.5 * Ly) - (dY > 0.5 * Ly));
  dX += gamma * dY;

  double a = aP * aP;
  double b = -(nxA * nxB + nyA * nyB);
  double c = aQ * aQ;
  double d = nxA * dX + nyA * dY;
  double e = -nxB * dX - nyB * dY;
  double delta = a * c - b * b;
  Recip64 iv{};
  if (FAST) iv = recip64(a, c, delta, sig);

  double t = fmin(fmax((FAST && delta > 0) ? (b * d - a * e) * iv.delta
                                            : (b * d - a * e) / delta,
                       -1.), 1.);
  double s = qdiv<FAST>(-(b * t + d), a, iv.a);
  double sarg = fabs(s);
  s = fmin(fmax(s, -1.), 1.);
  if (sarg > 1) t = fmin(fmax(qdiv<FAST>(-(b * s + e), c, iv.c), -1.), 1.);

  double dDx = dX + s * nxA - t * nxB;
  double dDy = dY + s * nyA - t * nyB;
  double dsq = dDx * dDx + dDy * dDy;
  if (!(dsq < sig * sig)) return false;
  double Fx, Fy, dij, dvij;
  if (FAST) {
    const double rs = rsqrt(dsq);
    dij = dsq * rs;
    dvij = (1.0 - dij * iv.sig) * iv.sig;
    Fx = dDx * (dvij * rs);
    Fy = dDy * (dvij * rs);
  } else {
    dij = sqrt(dsq);
    dvij = (1.0 - dij / sig) / sig;
    Fx = dDx * dvij / dij;
    Fy = dDy * dvij / dij;
  }
  o.fx = Fx;
  o.fy = Fy;
  o.tp = s * nxA * Fy - s * nyA * Fx;
  o.tq = t * nyB * Fx - t * nxB * Fy;
  if (SE && FAST) {
    const double CxA = s * nxA - 0.5 * dDx, CyA = s * nyA - 0.5 * dDy;
    const double CxB = t * nxB + 0.5 * dDx;
    const double CyB = (virial ? t * nyB : t * nxB) + 0.5 * dDy;
    const double gx = Fx * inv_LL, gy = Fy * inv_LL;
    o.e = dvij * sig * (1.0 - dij * iv.sig) * inv_two_n;
    if (!virial) {  // the reference's slips, as below
      o.pxx = gx * (CxA - CxB) - gy * CxB;
      o.pyy = gy * (CyA - CyB);
      o.pxy = gy * CxA;
      o.pyx = gx * (CyA - CyB);
    } else {
      o.pxx = gx * (CxA - CxB);
      o.pyy = gy * (CyA - CyB);
      o.pxy = gy * (CxA - CxB);
      o.pyx = gx * (CyA - CyB);
    }
  } else if (SE) {
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

// dX, dY: displacement P - Q already reduced to the minimum image (FP32);
// a = |u_A|^2 and c = |u_B|^2 are the squared half shaft lengths.
template <bool SE>
__device__ __forceinline__ bool pair_fp32(float dX, float dY, float nxA, float nyA, float a,
                                          float nxB, float nyB, float c, float sig, float gamma,
                                          bool virial, PairF32& o) {
  dX = fmaf(gamma, dY, dX);
  float b = -(nxA * nxB + nyA * nyB);
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
  float inv_sig = __fdividef(1.f, sig);
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

// Conservative FP32 screen: false only when the two spines (P at the origin, Q at
// -D in the sheared, minimum-image frame) are certainly farther apart than sig.
// The closest-point parameters come from the cross-product form; an error in them
// only moves the evaluated point pair along the spines, which can only raise the
// distance by the spines' misalignment angle times their length, and both that and
// the FP32 rounding of the distance stay far below the 1e-4 relative margin.  Both
// contact rules need the minimum distance below sig for any contact.
__device__ __forceinline__ bool may_touch_fp32(float dX, float dY, float nxA, float nyA,
                                               float aP, float nxB, float nyB, float aQ,
                                               float sig) {
  float a = aP * aP, c = aQ * aQ;
  float b = -(nxA * nxB + nyA * nyB);
  float d = nxA * dX + nyA * dY;
  float e = -(nxB * dX + nyB * dY);
  float w = nyA * nxB;
  float uxv = fmaf(nxA, nyB, -w) + fmaf(-nyA, nxB, w);
  float w2 = nyA * dX;
  float uxD = fmaf(nxA, dY, -w2) + fmaf(-nyA, dX, w2);
  float t = uxv == 0.f ? -1.f : fminf(fmaxf(__fdividef(uxD, uxv), -1.f), 1.f);
  float s = a > 0.f ? -__fdividef(b * t + d, a) : 0.f;
  float sarg = fabsf(s);
  s = fminf(fmaxf(s, -1.f), 1.f);
  if (sarg > 1.f && c > 0.f) t = fminf(fmaxf(-__fdividef(b * s + e, c), -1.f), 1.f);
  float dDx = dX + s * nxA - t * nxB;
  float dDy = dY + s * nyA - t * nyB;
  float lim = sig * 1.0001f + 1e-5f;
  return dDx * dDx + dDy * dDy < lim * lim;
}

// Spines P + s u_A and Q + t u_B (P - Q = D, lab frame) closer than lim: the
// closest points in FP32 with the cross-product form of the parameter (an error in
// it only moves the evaluated pair along the spines, raising the distance by the
// misalignment angle times the spine length, far below the caller's margin).
__device__ __forceinline__ bool capsules_within(float dX, float dY, float nxA, float nyA,
                                                float nxB, float nyB, float lim) {
  const float a = fmaf(nxA, nxA, nyA * nyA), c = fmaf(nxB, nxB, nyB * nyB);
  const float b = -(nxA * nxB + nyA * nyB);
  const float d = nxA * dX + nyA * dY;
  const float e = -(nxB * dX + nyB * dY);
  const float w = nyA * nxB;
  const float uxv = fmaf(nxA, nyB, -w) + fmaf(-nyA, nxB, w);
  const float w2 = nyA * dX;
  const float uxD = fmaf(nxA, dY, -w2) + fmaf(-nyA, dX, w2);
  float t = uxv == 0.f ? -1.f : fminf(fmaxf(__fdividef(uxD, uxv), -1.f), 1.f);
  float s = a > 0.f ? -__fdividef(b * t + d, a) : 0.f;
  const float sarg = fabsf(s);
  s = fminf(fmaxf(s, -1.f), 1.f);
  if (sarg > 1.f && c > 0.f) t = fminf(fmaxf(-__fdividef(b * s + e, c), -1.f), 1.f);
  const float x = dX + s * nxA - t * nxB, y = dY + s * nyA - t * nyB;
  return x * x + y * y < lim * lim;
}

// ---- two-point contacts (src/cuda/2point_dynamics.cu:385-546, euler_est_2p) ----
//
// For nearly parallel overlapping spines the single closest-point pair jumps from
// one end of the overlap to the other as the relative angle changes sign, which
// puts a cusp in the energy at alignment.  The reference's jamming code adds a
// second contact at the other end of the overlap (the closer of two candidates),
// each contact carrying its own harmonic overlap energy.  These functions return
// the spine parameters of both contacts in the reference's case analysis; has2 is
// false when the second candidate coincides with the first.
template <class T>
struct Contacts2 {
  T s1, t1, s2, t2;
  bool has2;
};

template <bool FAST = false>
__device__ __forceinline__ Contacts2<double> contacts2_fp64(double a, double b, double c, double d,
                                                            double e, double delta, double dX,
                                                            double dY, double nxA, double nyA,
                                                            double nxB, double nyB,
                                                            const Recip64& iv = Recip64{}) {
  double s1, t1, s2, t2, s3, t3;
  if (delta <= 0) {
    s1 = fmin(fmax(qdiv<FAST>(-(b + d), a, iv.a), -1.0), 1.0);
    s2 = fmin(fmax(qdiv<FAST>(-(d - b), a, iv.a), -1.0), 1.0);
    if (fabs(s1) == 1)
      t1 = fmin(fmax(qdiv<FAST>(-(b * s1 + e), c, iv.c), -1.0), 1.0);
    else if (b < 0)
      t1 = fmin(fmax(qdiv<FAST>(-(b + e), c, iv.c), -1.0), 1.0);
    else
      t1 = fmin(fmax(qdiv<FAST>(-(e - b), c, iv.c), -1.0), 1.0);
    if (fabs(s2) == 1)
      t2 = fmin(fmax(qdiv<FAST>(-(b * s2 + e), c, iv.c), -1.0), 1.0);
    else if (b < 0)
      t2 = fmin(fmax(qdiv<FAST>(-(e - b), c, iv.c), -1.0), 1.0);
    else
      t2 = fmin(fmax(qdiv<FAST>(-(b + e), c, iv.c), -1.0), 1.0);
    s3 = s2;
    t3 = t2;
  } else {
    t1 = fmin(fmax(qdiv<FAST>(b * d - a * e, delta, iv.delta), -1.), 1.);
    s1 = qdiv<FAST>(-(b * t1 + d), a, iv.a);
    double sarg = fabs(s1);
    s1 = fmin(fmax(s1, -1.), 1.);
    if (sarg >= 1) {
      t1 = fmin(fmax(qdiv<FAST>(-(b * s1 + e), c, iv.c), -1.), 1.);
      s2 = -s1;
      t2 = qdiv<FAST>(-(b * s2 + e), c, iv.c);
      double targ = fabs(t2);
      t2 = fmin(fmax(t2, -1.), 1.);
      if (targ > 1) {
        s2 = fmin(fmax(qdiv<FAST>(-(b * t2 + d), a, iv.a), -1.), 1.);
        s3 = s2;
        t3 = t2;
      } else {
        t3 = b < 0 ? -s1 : s1;
        s3 = qdiv<FAST>(-(b * t3 + d), a, iv.a);
        sarg = fabs(s3);
        s3 = fmin(fmax(s3, -1.0), 1.0);
        if (sarg >= 1) t3 = fmin(fmax(qdiv<FAST>(-(b * s3 + e), c, iv.c), -1.0), 1.0);
      }
    } else {
      t2 = -t1;
      s2 = qdiv<FAST>(-(b * t2 + d), a, iv.a);
      sarg = fabs(s2);
      s2 = fmin(fmax(s2, -1.), 1.);
      if (sarg > 1) {
        t2 = fmin(fmax(qdiv<FAST>(-(b * s2 + e), c, iv.c), -1.), 1.);
        s3 = s2;
        t3 = t2;
      } else {
        s3 = b < 0 ? -t1 : t1;
        t3 = qdiv<FAST>(-(b * s3 + e), c, iv.c);
        double targ = fabs(t3);
        t3 = fmin(fmax(t3, -1.0), 1.0);
        if (targ >= 1) s3 = fmin(fmax(qdiv<FAST>(-(b * t3 + d), a, iv.a), -1.0), 1.0);
      }
    }
  }
  Contacts2<double> r;
  r.s1 = s1;
  r.t1 = t1;
  r.has2 = (s1 != s2 && t1 != t2);
  if (r.has2 && s3 != s1 && s3 != s2) {
    double x2 = dX + s2 * nxA - t2 * nxB, y2 = dY + s2 * nyA - t2 * nyB;
    double x3 = dX + s3 * nxA - t3 * nxB, y3 = dY + s3 * nyA - t3 * nyB;
    if (x3 * x3 + y3 * y3 < x2 * x2 + y2 * y2) {
      s2 = s3;
      t2 = t3;
    }
  }
  r.s2 = s2;
  r.t2 = t2;
  return r;
}

// One harmonic contact at spine parameters (s, t); accumulates into o (no SE arms
// beyond the virial form: the two-point model is the reference's jamming path).
template <bool SE, bool FAST = false>
__device__ __forceinline__ bool contact_fp64(double dX, double dY, double s, double t, double nxA,
                                             double nyA, double nxB, double nyB, double sig,
                                             double LL, double two_n, PairF64& o,
                                             double inv_sig = 0.0, double inv_LL = 0.0,
                                             double inv_two_n = 0.0) {
  double dDx = dX + s * nxA - t * nxB;
  double dDy = dY + s * nyA - t * nyB;
  double dsq = dDx * dDx + dDy * dDy;
  if (!(dsq < sig * sig)) return false;
  double dij, dvij, Fx, Fy;
  if (FAST) {
    const double rs = rsqrt(dsq);
    dij = dsq * rs;
    dvij = (1.0 - dij * inv_sig) * inv_sig;
    Fx = dDx * (dvij * rs);
    Fy = dDy * (dvij * rs);
  } else {
    dij = sqrt(dsq);
    dvij = (1.0 - dij / sig) / sig;
    Fx = dDx * dvij / dij;
    Fy = dDy * dvij / dij;
  }
  o.fx += Fx;
  o.fy += Fy;
  o.tp += s * nxA * Fy - s * nyA * Fx;
  o.tq += t * nyB * Fx - t * nxB * Fy;
  if (SE && FAST) {
    const double CxA = s * nxA - 0.5 * dDx, CyA = s * nyA - 0.5 * dDy;
    const double CxB = t * nxB + 0.5 * dDx, CyB = t * nyB + 0.5 * dDy;
    const double gx = Fx * inv_LL, gy = Fy * inv_LL;
    o.e += dvij * sig * (1.0 - dij * inv_sig) * inv_two_n;
    o.pxx += gx * (CxA - CxB);
    o.pyy += gy * (CyA - CyB);
    o.pxy += gy * (CxA - CxB);
    o.pyx += gx * (CyA - CyB);
  } else if (SE) {
    double CxA = s * nxA - 0.5 * dDx, CyA = s * nyA - 0.5 * dDy;
    double CxB = t * nxB + 0.5 * dDx, CyB = t * nyB + 0.5 * dDy;
    o.e += dvij * sig * (1.0 - dij / sig) / two_n;
    o.pxx += Fx * CxA / LL - Fx * CxB / LL;
    o.pyy += Fy * CyA / LL - Fy * CyB / LL;
    o.pxy += Fy * CxA / LL - Fy * CxB / LL;
    o.pyx += Fx * CyA / LL - Fx * CyB / LL;
  }
  return true;
}

// Two-point contact pair in FP64 (minimum image and Lees-Edwards shift applied
// here, as in pair_fp64).  Stress uses the virial arms.
template <bool SE, bool FAST = false>
__device__ __forceinline__ bool pair2_fp64(double dX, double dY, double nxA, double nyA,
                                           double aP, double nxB, double nyB, double aQ,
                                           double sig, double gamma, double Lx, double Ly,
                                           double two_n, PairF64& o, double inv_LL = 0.0,
                                           double inv_two_n = 0.0) {
  dX += Lx * (double)((dX < -0.5 * Lx) - (dX > 0.5 * Lx));
  dY += Ly * (double)((dY < -0.5 * Ly) - (dY > 0.5 * Ly));
  dX += gamma * dY;
  double a = aP * aP;
  double b = -(nxA * nxB + nyA * nyB);
  double c = aQ * aQ;
  double d = nxA * dX + nyA * dY;
  double e = -nxB * dX - nyB * dY;
  double delta = a * c - b * b;
  Recip64 iv{};
  if (FAST) iv = recip64(a, c, delta, sig);
  Contacts2<double> k =
      contacts2_fp64<FAST>(a, b, c, d, e, delta, dX, dY, nxA, nyA, nxB, nyB, iv);
  o.fx = o.fy = o.tp = o.tq = 0.0;
  o.e = o.pxx = o.pyy = o.pxy = o.pyx = 0.0;
  const double LL = Lx * Ly;
  bool hit = contact_fp64<SE, FAST>(dX, dY, k.s1, k.t1, nxA, nyA, nxB, nyB, sig, LL, two_n, o,
                                    iv.sig, inv_LL, inv_two_n);
  if (k.has2)
    hit |= contact_fp64<SE, FAST>(dX, dY, k.s2, k.t2, nxA, nyA, nxB, nyB, sig, LL, two_n, o,
                                  iv.sig, inv_LL, inv_two_n);
  return hit;
}

// Two-point contact pair in FP32 on a displacement already reduced to the minimum
// image (as pair_fp32); the primary parameter uses the cross-product form.
__device__ __forceinline__ bool contact_fp32(float dX, float dY, float s, float t, float nxA,
                                             float nyA, float nxB, float nyB, float sig,
                                             PairF32& o) {
  float dDx = dX + s * nxA - t * nxB;
  float dDy = dY + s * nyA - t * nyB;
  float dsq = dDx * dDx + dDy * dDy;
  if (!(dsq < sig * sig)) return false;
  float inv_d = rsqrtf(dsq);
  float inv_sig = __fdividef(1.f, sig);
  float ov = 1.f - dsq * inv_d * inv_sig;
  float f = ov * inv_sig * inv_d;
  float Fx = dDx * f, Fy = dDy * f;
  o.fx += Fx;
  o.fy += Fy;
  o.tp += s * (nxA * Fy - nyA * Fx);
  o.tq += t * (nyB * Fx - nxB * Fy);
  o.ov += ov * ov;  // sum of squared overlaps of the contacts
  // stress: virial arms summed over the contacts, as force-weighted terms
  o.cxa += Fx * (s * nxA - 0.5f * dDx - t * nxB - 0.5f * dDx);
  o.cya += Fy * (s * nyA - 0.5f * dDy - t * nyB - 0.5f * dDy);
  o.cxb += Fy * (s * nxA - 0.5f * dDx - t * nxB - 0.5f * dDx);
  o.cyb += Fx * (s * nyA - 0.5f * dDy - t * nyB - 0.5f * dDy);
  return true;
}

// For the two-point model the PairF32 fields ov, cxa, cya, cxb, cyb hold summed
// quantities: sum ov^2, and the force-weighted virial terms Pxx, Pyy, Pxy, Pyx (before
// the division by the box area).
__device__ __forceinline__ bool pair2_fp32(float dX, float dY, float nxA, float nyA, float a,
                                           float nxB, float nyB, float c, float sig, float gamma,
                                           PairF32& o) {
  dX = fmaf(gamma, dY, dX);
  float b = -(nxA * nxB + nyA * nyB);
  float d = nxA * dX + nyA * dY;
  float e = -(nxB * dX + nyB * dY);
  float w = nyA * nxB;
  float uxv = fmaf(nxA, nyB, -w) + fmaf(-nyA, nxB, w);
  float w2 = nyA * dX;
  float uxD = fmaf(nxA, dY, -w2) + fmaf(-nyA, dX, w2);
  float s1, t1, s2, t2, s3, t3;
  auto cl = [](float v) { return fminf(fmaxf(v, -1.f), 1.f); };
  if (uxv == 0.f) {
    s1 = cl(-__fdividef(b + d, a));
    s2 = cl(-__fdividef(d - b, a));
    if (fabsf(s1) == 1.f)
      t1 = cl(-__fdividef(b * s1 + e, c));
    else
      t1 = cl(b < 0.f ? -__fdividef(b + e, c) : -__fdividef(e - b, c));
    if (fabsf(s2) == 1.f)
      t2 = cl(-__fdividef(b * s2 + e, c));
    else
      t2 = cl(b < 0.f ? -__fdividef(e - b, c) : -__fdividef(b + e, c));
    s3 = s2;
    t3 = t2;
  } else {
    t1 = cl(__fdividef(uxD, uxv));
    s1 = -__fdividef(b * t1 + d, a);
    float sarg = fabsf(s1);
    s1 = cl(s1);
    if (sarg >= 1.f) {
      t1 = cl(-__fdividef(b * s1 + e, c));
      s2 = -s1;
      t2 = -__fdividef(b * s2 + e, c);
      float targ = fabsf(t2);
      t2 = cl(t2);
      if (targ > 1.f) {
        s2 = cl(-__fdividef(b * t2 + d, a));
        s3 = s2;
        t3 = t2;
      } else {
        t3 = b < 0.f ? -s1 : s1;
        s3 = -__fdividef(b * t3 + d, a);
        sarg = fabsf(s3);
        s3 = cl(s3);
        if (sarg >= 1.f) t3 = cl(-__fdividef(b * s3 + e, c));
      }
    } else {
      t2 = -t1;
      s2 = -__fdividef(b * t2 + d, a);
      sarg = fabsf(s2);
      s2 = cl(s2);
      if (sarg > 1.f) {
        t2 = cl(-__fdividef(b * s2 + e, c));
        s3 = s2;
        t3 = t2;
      } else {
        s3 = b < 0.f ? -t1 : t1;
        t3 = -__fdividef(b * s3 + e, c);
        float targ = fabsf(t3);
        t3 = cl(t3);
        if (targ >= 1.f) s3 = cl(-__fdividef(b * t3 + d, a));
      }
    }
  }
  o.fx = o.fy = o.tp = o.tq = 0.f;
  o.ov = o.cxa = o.cya = o.cxb = o.cyb = 0.f;
  bool hit = contact_fp32(dX, dY, s1, t1, nxA, nyA, nxB, nyB, sig, o);
  if (s1 != s2 && t1 != t2) {
    if (s3 != s1 && s3 != s2) {
      float x2 = dX + s2 * nxA - t2 * nxB, y2 = dY + s2 * nyA - t2 * nyB;
      float x3 = dX + s3 * nxA - t3 * nxB, y3 = dY + s3 * nyA - t3 * nyB;
      if (x3 * x3 + y3 * y3 < x2 * x2 + y2 * y2) {
        s2 = s3;
        t2 = t3;
      }
    }
    hit |= contact_fp32(dX, dY, s2, t2, nxA, nyA, nxB, nyB, sig, o);
  }
  return hit;
}

// isolated_rotation, src/cpp/strain_dynamics.cpp:174-177
__device__ __forceinline__ double iso_rot64(double RC, double phi) {
  return 0.5 * (1 - RC * cos(2 * phi));
}

__device__ __forceinline__ int wrap_index(int v, int n) {
  return v < 0 ? v + n : (v >= n ? v - n : v);
}

}  // namespace sc
