// sc_fire.cu -- the production energy minimiser (FIRE) and the affine rescale used
// by quasistatic compression.
//
// The reference minimises with fixed-step gradient descent on the CPU
// (gradient_descent_minimize, tmarschall/spherocyls src/cpp/relaxation_dynamics.cpp:33-85,
// kept here step for step as sc_gd_minimize) and with a Polak-Ribiere conjugate
// gradient whose line search makes a host round trip per probe on the GPU
// (cjpr_relax_step_2p, src/cuda/2point_dynamics.cu:3886-4020).  Here the minimiser
// is FIRE (Bitzek et al., Phys. Rev. Lett. 97, 170201 (2006)), entirely on the
// device: each iteration is a force pass, a deterministic per-system reduction of
// F.v, |v|^2, |F|^2 and max |F|, a per-system scalar update, and a particle update,
// so a whole batch of packings minimises without any host synchronisation until
// the host polls the per-system "done" flags between chunks of iterations.
//
// Degrees of freedom (x, y, phi) with generalised forces (Fx, Fy, tau) and masses
// (1, 1, I); a system is done when every |F_i| and |tau_i|/sqrt(I_i) is below ftol.
#include "sc_internal.hpp"
#include "sc_pair.cuh"

namespace sc {

namespace {

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  float y = v + c;
  float t = s + y;
  c = y - (t - s);
  s = t;
}

// per-particle reduction terms of one chunk -> chunk partials (fixed order)
__global__ void k_fire_chunk(Dev d, FireState f) {
  int ch = blockIdx.x;
  if (f.sys[d.pchunk_sys[ch]].done) return;  // converged: its partials are not read
  int p0 = d.pchunk_p0[ch], np = d.pchunk_np[ch];
  double P = 0, vv = 0, ff = 0, fm = 0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) {
    int i = p0 + k;
    double I = d.irc[i].x;
    double fx = d.fx[i], fy = d.fy[i], tq = d.tau[i];
    double vx = f.vx[i], vy = f.vy[i], vp = f.vp[i];
    P += fx * vx + fy * vy + tq * vp;
    vv += vx * vx + vy * vy + I * vp * vp;
    ff += fx * fx + fy * fy + tq * tq / I;
    double m = fmax(fx * fx + fy * fy, tq * tq / I);
    fm = fmax(fm, m);
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

// FIRE scalar update of each system (Bitzek et al. 2006, parameters of that paper)
__global__ void k_fire_sys(Dev d, FireState f, double ftol, double dt_max) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.nsys) return;
  FireSys& q = f.sys[s];
  if (q.done) return;
  double P = 0, vv = 0, ff = 0, fm = 0;
  for (int ch = 0; ch < d.npchunks; ch++)
    if (d.pchunk_sys[ch] == s) {
      P += f.part[4 * ch + 0];
      vv += f.part[4 * ch + 1];
      ff += f.part[4 * ch + 2];
      fm = fmax(fm, f.part[4 * ch + 3]);
    }
  q.fmax = sqrt(fm);
  q.iters += 1;
  if (q.fmax < ftol) {
    q.done = 1;
    f.done[s] = 1;  // its force passes stop from the next iteration
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

// v <- (1-a) v + a |v| F/|F| (or 0 after an uphill step); v += dt F/m; x += dt v
__global__ void k_fire_update(Dev d, FireState f, int mixed) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  int s = d.psys[i];
  const FireSys q = f.sys[s];
  if (q.done) return;
  const SysGeom& g = d.geom[s];
  double I = d.irc[i].x;
  double fx = d.fx[i], fy = d.fy[i], tq = d.tau[i];
  double vx = f.vx[i], vy = f.vy[i], vp = f.vp[i];
  if (q.zero_v) {
    vx = vy = vp = 0.0;
  } else {
    vx = q.c1 * vx + q.c2 * fx;
    vy = q.c1 * vy + q.c2 * fy;
    vp = q.c1 * vp + q.c2 * tq / I;
  }
  vx += q.dt * fx;
  vy += q.dt * fy;
  vp += q.dt * tq / I;
  f.vx[i] = vx;
  f.vy[i] = vy;
  f.vp[i] = vp;
  double ddx = q.dt * vx, ddy = q.dt * vy, ddp = q.dt * vp;
  if (mixed) {
    float4 r = d.rec[i];
    float4 c = d.mc[i];
    kahan_add(r.x, c.x, (float)ddx);
    kahan_add(r.y, c.y, (float)ddy);
    kahan_add(c.z, c.w, (float)ddp);
    float sn, cs;
    sincosf(c.z + c.w, &sn, &cs);
    float A = d.pa[i].y;
    r.z = A * cs;
    r.w = A * sn;
    d.rec[i] = r;
    d.mc[i] = c;
    float4 m = d.mm[i];
    m.x += (float)ddx;
    m.y += (float)ddy;
    d.mm[i] = m;
    // the mixed list criterion (fixed gamma): spine movement since the build
    // (centre plus A times the rotation) and the next step's allowance within half
    // the padding
    float dd = (float)sqrt(ddx * ddx + ddy * ddy) + A * (float)fabs(ddp);
    float moved = sqrtf(m.x * m.x + m.y * m.y) + A * fabsf((c.z + c.w) - m.z);
    if (!(moved + dd < 0.5f * g.fpad)) {
      if (d.flags[s] == 0) atomicOr(&d.flags[s], 1);
      if (*d.any == 0) atomicExch(d.any, 1);
    }
  } else {
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

__global__ void k_fire_reset(Dev d, FireState f, double dt0) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ntot) {
    f.vx[i] = 0.0;
    f.vy[i] = 0.0;
    f.vp[i] = 0.0;
  }
  if (i < d.nsys) {
    FireSys q;
    q.dt = dt0;
    q.alpha = 0.1;
    q.c1 = 1.0;
    q.c2 = 0.0;
    q.fmax = 0.0;
    q.npos = 0;
    q.zero_v = 0;
    q.done = 0;
    q.iters = 0;
    f.sys[i] = q;
    f.done[i] = 0;
  }
}

// affine rescale of the FP64 positions: x by factor[2s], y by factor[2s+1] in system s
__global__ void k_affine(Dev d, const double* factor) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const int s = d.psys[i];
  const double fx = factor[2 * s], fy = factor[2 * s + 1];
  if (fx == 1.0 && fy == 1.0) return;
  double2 p = d.xy[i];
  d.xy[i] = make_double2(p.x * fx, p.y * fy);
}

// flip_shear_direction / reflect_yaxis (src/cuda/find_neighbors.cu:552-581):
// x -> Lx - x, phi -> -phi in the systems with lx[s] > 0
__global__ void k_reflect(Dev d, const double* lx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const double L = lx[d.psys[i]];
  if (!(L > 0)) return;
  double2 p = d.xy[i];
  d.xy[i] = make_double2(L - p.x, p.y);
  d.ph[i] = -d.ph[i];
}

// rotate_by_gamma / gamma_rotate (src/cuda/find_neighbors.cu:583-645) for the
// systems with q[4s+3] != 0: q[4s..4s+2] = (gamma, new Lx, new Ly).  Positions are
// mapped to the frame in which the sheared cell is upright (an isometry of the
// Lees-Edwards system), angles turned by atan(1/gamma), each wrapped once.
__global__ void k_rotate(Dev d, const double* q) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const int s = d.psys[i];
  if (q[4 * s + 3] == 0.0) return;
  const double g = q[4 * s], Lx = q[4 * s + 1], Ly = q[4 * s + 2];
  const double pi = 3.14159265358979;  // D_PI of the reference
  const double2 p = d.xy[i];
  const double sg = 1 - 2 * (double)signbit(g);
  const double root = sqrt(1 + g * g);
  double nx = sg * p.y * root;
  double ny = -sg * p.x / root;
  double phi = g != 0.0 ? d.ph[i] - atan(1 / g) : d.ph[i] - pi / 2;
  if (phi > pi)
    phi -= 2 * pi;
  else if (phi < -pi)
    phi += 2 * pi;
  if (ny > Ly)
    ny -= Ly;
  else if (ny < 0)
    ny += Ly;
  if (nx < 0)
    nx += Lx;
  else if (nx > Lx)
    nx -= Lx;
  d.xy[i] = make_double2(nx, ny);
  d.ph[i] = phi;
}

inline int nblk(int n, int b) { return (n + b - 1) / b; }

}  // namespace

void launch_fire_reset(const Dev& d, const FireState& f, double dt0, cudaStream_t st) {
  int n = d.ntot > d.nsys ? d.ntot : d.nsys;
  k_fire_reset<<<nblk(n, 256), 256, 0, st>>>(d, f, dt0);
}

void launch_fire_iteration_tail(const Dev& d, const FireState& f, double ftol, double dt_max,
                                bool mixed, cudaStream_t st) {
  k_fire_chunk<<<d.npchunks, 256, 0, st>>>(d, f);
  k_fire_sys<<<nblk(d.nsys, 128), 128, 0, st>>>(d, f, ftol, dt_max);
  k_fire_update<<<nblk(d.ntot, 256), 256, 0, st>>>(d, f, mixed ? 1 : 0);
}

void launch_rotate(const Dev& d, const double* q, cudaStream_t st) {
  k_rotate<<<nblk(d.ntot, 256), 256, 0, st>>>(d, q);
}

void launch_reflect(const Dev& d, const double* lx, cudaStream_t st) {
  k_reflect<<<nblk(d.ntot, 256), 256, 0, st>>>(d, lx);
}

void launch_affine(const Dev& d, const double* factor, cudaStream_t st) {
  k_affine<<<nblk(d.ntot, 256), 256, 0, st>>>(d, factor);
}

}  // namespace sc
