// sc_cg.cu -- the reference's Polak-Ribiere conjugate-gradient minimiser, with its
// line search, on the device.
//
// cjpr_relax_step_2p / line_search_2p (tmarschall/spherocyls
// src/cuda/2point_dynamics.cu:3609-3780, 3886-4020) make one host round trip per
// energy probe: the line search is a recursion on the host over energies read back
// from the GPU.  Here each system's line search is a state machine in device memory,
// advanced by one thread per system after every probe, and the probes run inside a
// CUDA-graph WHILE node that repeats while any system is still searching, so a
// batch of packings minimises without host synchronisation until the host polls
// the per-system "done" flags between chunks of iterations.
//
// One iteration (all systems at once, each kernel skipping finished systems):
//   forces and energy at x (force pass) -> |F|^2, F.F0, |F0|^2 (k_cg_dots) ->
//   stop tests, beta, initial step (k_cg_begin) -> D = F + beta D (k_cg_dir) ->
//   WHILE searching { x_t = x + t D (k_cg_probe); E(x_t) (energy pass);
//                     next t or the chosen step (k_cg_search) } ->
//   x += t_min step D, moved distance, rebuild request (k_cg_move).
// Generalised coordinates (x, y, phi) with forces (Fx, Fy, tau), as the reference
// (its square norms use the raw torque, square_forces_2p :3188-3239).
#include "sc_internal.hpp"

namespace sc {

namespace {

inline int nblk(int n, int b) { return (n + b - 1) / b; }

// per-particle terms of |F|^2, F.F0 and |F0|^2 -> chunk partials (fixed order)
__global__ void k_cg_dots(Dev d, CgState c) {
  const int ch = blockIdx.x;
  const int p0 = d.pchunk_p0[ch], np = d.pchunk_np[ch];
  double ff = 0, f0 = 0, oo = 0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) {
    const int i = p0 + k;
    const double fx = d.fx[i], fy = d.fy[i], tq = d.tau[i];
    const double ox = d.cg0x[i], oy = d.cg0y[i], op = d.cg0p[i];
    ff += fx * fx + fy * fy + tq * tq;
    f0 += fx * ox + fy * oy + tq * op;
    oo += ox * ox + oy * oy + op * op;
  }
  __shared__ double sh[3][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o; o >>= 1) {
    ff += __shfl_down_sync(0xffffffffu, ff, o);
    f0 += __shfl_down_sync(0xffffffffu, f0, o);
    oo += __shfl_down_sync(0xffffffffu, oo, o);
  }
  if (lane == 0) {
    sh[0][w] = ff;
    sh[1][w] = f0;
    sh[2][w] = oo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0, e = 0;
    for (int k = 0; k < nw; k++) {
      a += sh[0][k];
      b += sh[1][k];
      e += sh[2][k];
    }
    c.part[3 * ch + 0] = a;
    c.part[3 * ch + 1] = b;
    c.part[3 * ch + 2] = e;
  }
}

// Start of an iteration, one block per system (cjpr_relax_step_2p :3886-3946 and the
// restart of cjpr_relax_2p :4270-4274): the system's chunk partials summed in a fixed
// tree over the block, then, in one thread, the energy history and its stop tests,
// the Polak-Ribiere beta = max(0, (F.F - F.F0)/F0.F0), and the first line-search step
// 2e-6/|F|_rms within [1e-18, 2]/|F|_rms.  `search` is the WHILE node of this
// iteration's line search (switched on when any system starts one).
constexpr int kCgBlock = 256;
__global__ void __launch_bounds__(kCgBlock) k_cg_begin(Dev d, CgState c, int max_iter,
                                                       unsigned long long search) {
  const int s = blockIdx.x;
  CgSys& q = c.sys[s];
  if (q.done) return;  // block-uniform
  double F2 = 0, FF0 = 0, F02 = 0;
  const int ch0 = d.geom[s].pch0, ch1 = ch0 + pchunk_count(d.geom[s]);
  for (int ch = ch0 + (int)threadIdx.x; ch < ch1; ch += kCgBlock) {
    F2 += c.part[3 * ch + 0];
    FF0 += c.part[3 * ch + 1];
    F02 += c.part[3 * ch + 2];
  }
  __shared__ double sh[3][kCgBlock / 32];
  for (int o = 16; o; o >>= 1) {
    F2 += __shfl_down_sync(0xffffffffu, F2, o);
    FF0 += __shfl_down_sync(0xffffffffu, FF0, o);
    F02 += __shfl_down_sync(0xffffffffu, F02, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = F2;
    sh[1][threadIdx.x >> 5] = FF0;
    sh[2][threadIdx.x >> 5] = F02;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  F2 = FF0 = F02 = 0.0;
  for (int k = 0; k < kCgBlock / 32; k++) {
    F2 += sh[0][k];
    FF0 += sh[1][k];
    F02 += sh[2][k];
  }
  q.Eh2 = q.Eh1;
  q.Eh1 = q.E0;
  q.E0 = d.se_sys[s];  // se_sys is [5][nsys]: the energies come first
  q.F2 = F2;
  if (F2 == 0) {  // "Zero energy found"
    q.done = 1;
    q.reason = CG_ZERO_FORCE;
    return;
  }
  if (q.Eh1 == q.E0 && q.Eh2 == q.Eh1) {  // "Minimum Energy Found"
    q.done = 1;
    q.reason = CG_STALLED;
    return;
  }
  if (q.iters >= max_iter) {
    q.done = 1;
    q.reason = CG_MAX_ITER;
    return;
  }
  q.iters += 1;
  const int n = d.geom[s].n;
  // the direction starts from F, and again every 3N iterations
  const bool restart = (q.iters - 1) % (3 * n) == 0;
  q.beta = (restart || !(F02 > 0)) ? 0.0 : fmax(0.0, (F2 - FF0) / F02);
  q.norm = sqrt(F2 / (3 * n));
  q.step = 2e-6 / q.norm;
  q.min_step = 1e-18 / q.norm;
  q.max_step = 2 / q.norm;
  q.attempt = 0;
  q.redirect = 0;
  q.probes = 0;
  q.t = q.step;
  q.phase = CG_TOP;
  *c.searching = 1;
  if (search) cudaGraphSetConditional(search, 1u);
}

// D = F + beta D for the systems starting a line search; F0 = F for the next beta
__global__ void k_cg_dir(Dev d, CgState c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const CgSys& q = c.sys[d.psys[i]];
  if (q.done || q.phase != CG_TOP) return;
  const double fx = d.fx[i], fy = d.fy[i], tq = d.tau[i];
  d.fvx[i] = fx + q.beta * d.fvx[i];
  d.fvy[i] = fy + q.beta * d.fvy[i];
  d.fvp[i] = tq + q.beta * d.fvp[i];
  d.cg0x[i] = fx;
  d.cg0y[i] = fy;
  d.cg0p[i] = tq;
}

// The probe x_t = x + t D of each searching system (temp_move_step_2p :3381-3405),
// after a direction change the failed search asked for: D = F (steepest descent), or
// D = F/sqrt(|F|) per particle (sqrt_grad_dir_2p :3293-3340).
__global__ void k_cg_probe(Dev d, CgState c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const CgSys& q = c.sys[d.psys[i]];
  if (q.done || q.phase < CG_TOP || q.phase > CG_FINAL) return;
  double dx, dy, dp;
  if (q.redirect == 1) {
    dx = d.fx[i];
    dy = d.fy[i];
    dp = d.tau[i];
    d.fvx[i] = dx;
    d.fvy[i] = dy;
    d.fvp[i] = dp;
  } else if (q.redirect == 2) {
    const double fx = d.fx[i], fy = d.fy[i], tq = d.tau[i];
    const double fm = sqrt(fx * fx + fy * fy), tm = fabs(tq);
    dx = fm == 0 ? 0.0 : fx / sqrt(fm);
    dy = fm == 0 ? 0.0 : fy / sqrt(fm);
    dp = tm == 0 ? 0.0 : tq / sqrt(tm);
    d.fvx[i] = dx;
    d.fvy[i] = dy;
    d.fvp[i] = dp;
  } else {
    dx = d.fvx[i];
    dy = d.fvy[i];
    dp = d.fvp[i];
  }
  const double2 p = d.xy[i];
  const double pht = d.ph[i] + q.t * dp;
  d.xy_t[i] = make_double2(p.x + q.t * dx, p.y + q.t * dy);
  d.ph_t[i] = pht;
  const double A = d.ra[i].y;
  double sn, cs;
  sincos(pht, &sn, &cs);
  d.nxy_t[i] = make_double2(A * cs, A * sn);
}

// The parabola through (0, E0), (1, E1), (2, E2) in units of the step and its
// minimum, clipped at 2 (line_search_2p :3705-3711); the final probe comes next.
__device__ void cg_find_min(CgSys& q) {
  if (q.E1 > q.E0) {  // "Cannot find lower energy": another direction, or stop
    if (q.attempt == 0) {
      q.attempt = 1;
      q.redirect = 1;
      q.step = 1e-6 / q.norm;
      q.t = q.step;
      q.phase = CG_TOP;
    } else if (q.attempt == 1) {
      const double rn = sqrt(q.norm);
      q.attempt = 2;
      q.redirect = 2;
      q.step = 2e-6 / rn;
      q.min_step = 1e-18 / rn;
      q.max_step = 2 / rn;
      q.t = q.step;
      q.phase = CG_TOP;
    } else {
      q.phase = CG_IDLE;  // "Stopping due to step size"
      q.done = 1;
      q.reason = CG_STEP;
    }
    return;
  }
  double tmin = (3 * q.E0 - 4 * q.E1 + q.E2) / (2 * q.E0 - 4 * q.E1 + 2 * q.E2);
  if (tmin > 2)
    tmin = 2;
  else if (q.E1 == q.E0)
    tmin = 1;
  q.tmin = tmin;
  q.t = tmin * q.step;
  q.phase = CG_FINAL;
}

// One transition of each searching system's line search on the energy of its last
// probe (line_search_2p :3609-3780 as a flat state machine: TOP probes the step,
// SECOND twice the step, HALVE and DOUBLE are the reference's recursive calls with
// (first, second) = (1, 0) and (0, 1), FINAL the parabola's minimum).  `search` is
// switched off when no system probes again.  The halvings and doublings are bounded
// by the step limits (about 45 probes per direction attempt, three attempts), and a
// search that still asks for another probe after c.max_probes ends its system with
// reason CG_PROBES, so the WHILE node ends whatever the energies do.
__global__ void k_cg_search(Dev d, CgState c, unsigned long long search) {
  bool again = false;
  for (int s = threadIdx.x; s < d.nsys; s += blockDim.x) {
    CgSys& q = c.sys[s];
    if (!q.done && q.phase >= CG_TOP && q.phase <= CG_FINAL) {
      const double E = d.se_sys[s];
      q.redirect = 0;
      switch (q.phase) {
        case CG_TOP:
          q.E1 = E;
          if (q.E1 > q.E0 && q.step > q.min_step) {
            q.step /= 2;
            q.E2 = q.E1;
            q.t = q.step;
            q.phase = CG_HALVE;
          } else {
            q.t = 2 * q.step;
            q.phase = CG_SECOND;
          }
          break;
        case CG_HALVE:
          q.E1 = E;
          if (q.E1 > q.E0 && q.step > q.min_step) {
            q.step /= 2;
            q.E2 = q.E1;
            q.t = q.step;
          } else {
            cg_find_min(q);
          }
          break;
        case CG_SECOND:
        case CG_DOUBLE:
          q.E2 = E;
          if (q.E2 <= q.E1 && q.step < q.max_step) {
            q.step *= 2;
            q.E1 = q.E2;
            q.t = 2 * q.step;
            q.phase = CG_DOUBLE;
          } else {
            cg_find_min(q);
          }
          break;
        case CG_FINAL:
          if (E > q.E1) q.tmin = 1;
          q.phase = CG_MOVE;
          break;
      }
      q.probes += 1;
      if (!q.done && q.phase >= CG_TOP && q.phase <= CG_FINAL && q.probes >= c.max_probes) {
        q.phase = CG_IDLE;
        q.done = 1;
        q.reason = CG_PROBES;
      }
      again = again || (!q.done && q.phase >= CG_TOP && q.phase <= CG_FINAL);
    }
  }
  // one block: the loop switch is decided once
  const int any = __syncthreads_or(again);
  if (search && threadIdx.x == 0) cudaGraphSetConditional(search, any ? 1u : 0u);
  if (threadIdx.x == 0) *c.searching = any;
}

// x += t_min step D for the systems whose search ended (move_step_2p :3412-3460),
// with the moved distance and the rebuild request of the src/cpp rule (a per-axis
// displacement beyond half the padding)
__global__ void k_cg_move(Dev d, CgState c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const int s = d.psys[i];
  const CgSys& q = c.sys[s];
  if (q.phase != CG_MOVE) return;
  const double h = q.tmin * q.step;
  const double ddx = h * d.fvx[i], ddy = h * d.fvy[i], ddp = h * d.fvp[i];
  double2 p = d.xy[i];
  p.x += ddx;
  p.y += ddy;
  const double phi = d.ph[i] + ddp;
  d.xy[i] = p;
  d.ph[i] = phi;
  const double A = d.ra[i].y;
  double sn, cs;
  sincos(phi, &sn, &cs);
  d.nxy[i] = make_double2(A * cs, A * sn);
  double2 m = d.moved[i];
  m.x += ddx;
  m.y += ddy;
  d.moved[i] = m;
  if (!(isfinite(p.x) && isfinite(p.y) && isfinite(phi))) atomicOr(d.status, ST_NAN);
  const double pad = d.geom[s].pad;
  if (m.x > 0.5 * pad || m.x < -0.5 * pad || m.y > 0.5 * pad || m.y < -0.5 * pad)
    request_rebuild(d, s);
}

// a finished move returns the system to the idle state (after k_cg_move); a rebuild
// still pending switches the rebuild node on as well
__global__ void k_cg_settle(Dev d, CgState c) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0 && d.cond && *d.any != 0) cudaGraphSetConditional(d.cond, 1u);
  if (s >= d.nsys) return;
  CgSys& q = c.sys[s];
  if (q.phase == CG_MOVE) q.phase = CG_IDLE;
}

__global__ void k_cg_reset(Dev d, CgState c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.ntot) {
    d.fvx[i] = 0.0;
    d.fvy[i] = 0.0;
    d.fvp[i] = 0.0;
    d.cg0x[i] = 0.0;
    d.cg0y[i] = 0.0;
    d.cg0p[i] = 0.0;
  }
  if (i < d.nsys) {
    CgSys q{};
    q.phase = CG_IDLE;
    c.sys[i] = q;
  }
}

}  // namespace

void launch_cg_reset(const Dev& d, const CgState& c, cudaStream_t st) {
  const int n = d.ntot > d.nsys ? d.ntot : d.nsys;
  k_cg_reset<<<nblk(n, 256), 256, 0, st>>>(d, c);
}

void launch_cg_begin(const Dev& d, const CgState& c, int max_iter, unsigned long long search,
                     cudaStream_t st) {
  k_cg_dots<<<d.npchunks, 256, 0, st>>>(d, c);
  k_cg_begin<<<d.nsys, kCgBlock, 0, st>>>(d, c, max_iter, search);
  k_cg_dir<<<nblk(d.ntot, 256), 256, 0, st>>>(d, c);
}

void launch_cg_probe(const Dev& d, const CgState& c, cudaStream_t st) {
  k_cg_probe<<<nblk(d.ntot, 256), 256, 0, st>>>(d, c);
}

void launch_cg_search(const Dev& d, const CgState& c, unsigned long long search,
                      cudaStream_t st) {
  k_cg_search<<<1, 1024, 0, st>>>(d, c, search);
}

void launch_cg_move(const Dev& d, const CgState& c, cudaStream_t st) {
  k_cg_move<<<nblk(d.ntot, 256), 256, 0, st>>>(d, c);
  k_cg_settle<<<nblk(d.nsys, 128), 128, 0, st>>>(d, c);
}

}  // namespace sc
