// sc_fire.cuh -- the steps of one FIRE iteration as device functions, shared by the
// launch-per-kernel form (sc_fire.cu) and the persistent form (sc_pass_mixed.cu),
// compiled with the same fused multiply-adds so that both give the same iterates.
//
// FIRE: Bitzek et al., Phys. Rev. Lett. 97, 170201 (2006).  Degrees of freedom
// (x, y, phi) with generalised forces (Fx, Fy, tau) and masses (1, 1, I); a system
// is done when every |F_i| and |tau_i|/sqrt(I_i) is below ftol.
#pragma once

#include "sc_internal.hpp"

namespace sc {
namespace fire {

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  float y = v + c;
  float t = s + y;
  c = y - (t - s);
  s = t;
}

// per-particle reduction terms of one chunk -> chunk partials (fixed order).  The
// mixed form's forces and velocities are FP32 values (held in the FP64 arrays): its
// per-particle products are FP32 and only the sums are FP64, which keeps the FP64
// pipe (a small fraction of the FP32 rate on this GPU) out of the per-particle work.
template <bool MIXED>
__device__ __forceinline__ void fire_chunk(const Dev& d, const FireState& f, int ch) {
  if (f.sys[d.pchunk_sys[ch]].done) return;  // converged: its partials are not read
  int p0 = d.pchunk_p0[ch], np = d.pchunk_np[ch];
  double P = 0, vv = 0, ff = 0, fm = 0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) {
    int i = p0 + k;
    if (MIXED) {
      const float fx = (float)d.fx[i], fy = (float)d.fy[i], tq = (float)d.tau[i];
      const float vx = (float)f.vx[i], vy = (float)f.vy[i], vp = (float)f.vp[i];
      const float invI = d.pa[i].w;  // FP32 1/I of the mixed records
      const float t2 = tq * tq * invI;
      const float f2 = fmaf(fx, fx, fy * fy);
      P += (double)fmaf(fx, vx, fmaf(fy, vy, tq * vp));
      vv += (double)fmaf(vx, vx, fmaf(vy, vy, __fdividef(vp * vp, invI)));
      ff += (double)(f2 + t2);
      fm = fmax(fm, (double)fmaxf(f2, t2));
    } else {
      double I = d.irc[i].x;
      double fx = d.fx[i], fy = d.fy[i], tq = d.tau[i];
      double vx = f.vx[i], vy = f.vy[i], vp = f.vp[i];
      const double t2 = tq * tq / I;  // one FP64 division per particle
      P += fx * vx + fy * vy + tq * vp;
      vv += vx * vx + vy * vy + I * vp * vp;
      ff += fx * fx + fy * fy + t2;
      double m = fmax(fx * fx + fy * fy, t2);
      fm = fmax(fm, m);
    }
  }
  __shared__ double sh[4][32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o; o >>= 1) {
    P += __shfl_down_sync(0xffffffffu, P, o);
    vv += __shfl_down_sync(0xffffffffu, vv, o);
    ff += __shfl_down_sync(0xffffffffu, ff, o);
    fm = fmax(fm, __shfl_down_sync(0xffffffffu, fm, o));
  }
  if (lane == 0) {
    sh[0][w] = P;
    sh[1][w] = vv;
    sh[2][w] = ff;
    sh[3][w] = fm;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0, c = 0, m = 0;
    for (int k = 0; k < nw; k++) {
      a += sh[0][k];
      b += sh[1][k];
      c += sh[2][k];
      m = fmax(m, sh[3][k]);
    }
    f.part[4 * ch + 0] = a;
    f.part[4 * ch + 1] = b;
    f.part[4 * ch + 2] = c;
    f.part[4 * ch + 3] = m;
  }
}

// The FIRE scalar update of one system from its sums F.v, |v|^2, |F|^2, max|F|^2.
__device__ __forceinline__ void fire_sys_scalars(FireSys& q, int* done_flag, double P, double vv,
                                                 double ff, double fm, double ftol,
                                                 double dt_max) {
  q.fmax = sqrt(fm);
  q.iters += 1;
  if (q.fmax < ftol) {
    q.done = 1;
    *done_flag = 1;  // its force passes stop from the next iteration
    q.c1 = 1.0;
    q.c2 = 0.0;
    q.dt = 0.0;
    return;
  }
  const double f_inc = 1.1, f_dec = 0.5, a_start = 0.1, f_a = 0.99;
  const int n_min = 5;
  q.c1 = 1.0 - q.alpha;
  q.c2 = ff > 0 ? q.alpha * sqrt(vv / ff) : 0.0;
  q.zero_v = 0;
  if (P > 0) {
    q.npos += 1;
    if (q.npos > n_min) {
      q.dt = fmin(q.dt * f_inc, dt_max);
      q.alpha *= f_a;
    }
  } else {
    q.npos = 0;
    q.dt *= f_dec;
    q.alpha = a_start;
    q.zero_v = 1;
  }
}

// FIRE scalar update of system s (Bitzek et al. 2006, parameters of that paper) by
// one block of kFireBlock threads: the system's chunk partials are summed in a fixed
// tree over the block (a large system has hundreds of chunks), then one thread
// updates the scalars.
constexpr int kFireBlock = 256;
__device__ __forceinline__ void fire_sys(const Dev& d, const FireState& f, int s, double ftol,
                                         double dt_max) {
  __shared__ double sh[4][kFireBlock / 32];
  if (f.sys[s].done) return;  // block-uniform
  double P = 0, vv = 0, ff = 0, fm = 0;
  const int ch0 = d.geom[s].pch0, ch1 = ch0 + pchunk_count(d.geom[s]);
  for (int ch = ch0 + (int)threadIdx.x; ch < ch1; ch += kFireBlock) {
    P += f.part[4 * ch + 0];
    vv += f.part[4 * ch + 1];
    ff += f.part[4 * ch + 2];
    fm = fmax(fm, f.part[4 * ch + 3]);
  }
  for (int o = 16; o; o >>= 1) {
    P += __shfl_down_sync(0xffffffffu, P, o);
    vv += __shfl_down_sync(0xffffffffu, vv, o);
    ff += __shfl_down_sync(0xffffffffu, ff, o);
    fm = fmax(fm, __shfl_down_sync(0xffffffffu, fm, o));
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][w] = P;
    sh[1][w] = vv;
    sh[2][w] = ff;
    sh[3][w] = fm;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    P = vv = ff = fm = 0.0;
    for (int k = 0; k < kFireBlock / 32; k++) {
      P += sh[0][k];
      vv += sh[1][k];
      ff += sh[2][k];
      fm = fmax(fm, sh[3][k]);
    }
    fire_sys_scalars(f.sys[s], f.done + s, P, vv, ff, fm, ftol, dt_max);
  }
  __syncthreads();  // sh is reused by the block's next system
}

// v <- (1-a) v + a |v| F/|F| (or 0 after an uphill step); v += dt F/m; x += dt v.
// The mixed form's velocity update is FP32 (its forces are FP32), stored in the
// FP64 arrays; the FP64 form's is FP64.
template <bool MIXED>
__device__ __forceinline__ void fire_update(const Dev& d, const FireState& f, int i) {
  int s = d.psys[i];
  const FireSys q = f.sys[s];
  if (q.done) return;
  const SysGeom& g = d.geom[s];
  if (MIXED) {
    const float4 pa = d.pa[i];  // (R, A, index bits, 1/I)
    const float A = pa.y;
    const float fx = (float)d.fx[i], fy = (float)d.fy[i], ap = (float)d.tau[i] * pa.w;
    float vx = (float)f.vx[i], vy = (float)f.vy[i], vp = (float)f.vp[i];
    const float c1 = (float)q.c1, c2 = (float)q.c2, dt = (float)q.dt;
    if (q.zero_v) {
      vx = vy = vp = 0.f;
    } else {
      vx = fmaf(c1, vx, c2 * fx);
      vy = fmaf(c1, vy, c2 * fy);
      vp = fmaf(c1, vp, c2 * ap);
    }
    vx = fmaf(dt, fx, vx);
    vy = fmaf(dt, fy, vy);
    vp = fmaf(dt, ap, vp);
    f.vx[i] = vx;
    f.vy[i] = vy;
    f.vp[i] = vp;
    const float ddx = dt * vx, ddy = dt * vy, ddp = dt * vp;
    float4 r = d.rec[i];
    float4 c = d.mc[i];
    kahan_add(r.x, c.x, ddx);
    kahan_add(r.y, c.y, ddy);
    kahan_add(c.z, c.w, ddp);
    float sn, cs;
    sincosf(c.z + c.w, &sn, &cs);
    r.z = A * cs;
    r.w = A * sn;
    d.rec[i] = r;
    d.mc[i] = c;
    float4 m = d.mm[i];
    m.x += ddx;
    m.y += ddy;
    d.mm[i] = m;
    // the mixed list criterion (fixed gamma): spine movement since the build
    // (centre plus A times the rotation) and the next step's allowance within half
    // the padding
    float dd = sqrtf(fmaf(ddx, ddx, ddy * ddy)) + A * fabsf(ddp);
    float moved = sqrtf(m.x * m.x + m.y * m.y) + A * fabsf((c.z + c.w) - m.z);
    if (!(moved + dd < 0.5f * g.fpad)) {
      if (d.flags[s] == 0) atomicOr(&d.flags[s], 1);
      if (*d.any == 0) atomicExch(d.any, 1);
    }
  } else {
    double I = d.irc[i].x;
    double fx = d.fx[i], fy = d.fy[i], tq = d.tau[i];
    double vx = f.vx[i], vy = f.vy[i], vp = f.vp[i];
    const double ap = tq / I;  // angular acceleration (one FP64 division)
    if (q.zero_v) {
      vx = vy = vp = 0.0;
    } else {
      vx = q.c1 * vx + q.c2 * fx;
      vy = q.c1 * vy + q.c2 * fy;
      vp = q.c1 * vp + q.c2 * ap;
    }
    vx += q.dt * fx;
    vy += q.dt * fy;
    vp += q.dt * ap;
    f.vx[i] = vx;
    f.vy[i] = vy;
    f.vp[i] = vp;
    double ddx = q.dt * vx, ddy = q.dt * vy, ddp = q.dt * vp;
    double2 p = d.xy[i];
    p.x += ddx;
    p.y += ddy;
    double phi = d.ph[i] + ddp;
    d.xy[i] = p;
    d.ph[i] = phi;
    double2 ra = d.ra[i];
    double sn, cs;
    sincos(phi, &sn, &cs);
    d.nxy[i] = make_double2(ra.y * cs, ra.y * sn);
    double2 m = d.moved[i];
    m.x += ddx;
    m.y += ddy;
    d.moved[i] = m;
    if (m.x > 0.5 * g.pad || m.x < -0.5 * g.pad || m.y > 0.5 * g.pad || m.y < -0.5 * g.pad) {
      if (d.flags[s] == 0) atomicOr(&d.flags[s], 1);
      if (*d.any == 0) atomicExch(d.any, 1);
    }
  }
}

}  // namespace fire
}  // namespace sc
