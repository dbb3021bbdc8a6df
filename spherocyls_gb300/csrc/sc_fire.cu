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
#include "sc_fire.cuh"
#include "sc_internal.hpp"
#include "sc_pair.cuh"

namespace sc {

namespace {

// one block per chunk
template <bool MIXED>
__global__ void k_fire_chunk(Dev d, FireState f) { fire::fire_chunk<MIXED>(d, f, blockIdx.x); }

// one block of fire::kFireBlock threads per system
__global__ void __launch_bounds__(fire::kFireBlock) k_fire_sys(Dev d, FireState f, double ftol,
                                                               double dt_max) {
  fire::fire_sys(d, f, blockIdx.x, ftol, dt_max);
}

template <bool MIXED>
__global__ void k_fire_update(Dev d, FireState f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ntot) fire::fire_update<MIXED>(d, f, i);
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
  if (mixed)
    k_fire_chunk<true><<<d.npchunks, 256, 0, st>>>(d, f);
  else
    k_fire_chunk<false><<<d.npchunks, 256, 0, st>>>(d, f);
  k_fire_sys<<<d.nsys, fire::kFireBlock, 0, st>>>(d, f, ftol, dt_max);
  if (mixed)
    k_fire_update<true><<<nblk(d.ntot, 256), 256, 0, st>>>(d, f);
  else
    k_fire_update<false><<<nblk(d.ntot, 256), 256, 0, st>>>(d, f);
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
