// sc_cells.cu -- cell-list build (counting sort of particles by cell), Lees-Edwards
// set-back, stress/energy reductions and the gradient-descent update.
//
// The rebuild follows the reference's find_cells / find_neighbors
// (tmarschall/spherocyls src/cpp/spherocyl_box.cpp:270-355): positions are wrapped
// into the box, each particle is hashed to its cell (col + row*cols in the
// reference; here numbered tile by tile, see cell_local), and the cell lists
// hold particles in increasing particle index.  On the GPU the lists are a
// counting sort of the particle arrays themselves into cell order:
//
//   zero counts -> hash (atomic rank inside the cell) -> per-chunk sums ->
//   per-system scan of chunk sums -> per-chunk scan = cell starts -> scatter ->
//   sort each cell's slots by particle index (makes the order deterministic and
//   equal to the reference's cell-list order) -> gather into scratch -> commit.
//
// Only systems whose flag is set are rebuilt; every kernel exits at once when no
// system is flagged, so the chain can sit in every step of a captured graph.
// Compiled with -fmad=false: the wrap arithmetic and the set-back are the
// reference's IEEE operations.
#include "sc_internal.hpp"
#include "sc_pair.cuh"

namespace sc {

namespace {

constexpr double kRefPi = 3.14159265358979;  // src/cpp/spherocyl_box.cpp:12

// The reference's wrap loops (while v > hi: v -= period; while v < lo: v += period).
// A runaway value would make them spin for ever; after 64 periods the wrap
// finishes with floor() and flags the state as non-finite instead.
__device__ __forceinline__ double wrap_bounded(double v, double lo, double hi, double period,
                                               int* status) {
  int it = 0;
  while (v > hi && it < 64) {
    v -= period;
    it++;
  }
  while (v < lo && it < 64) {
    v += period;
    it++;
  }
  if (it >= 64) {
    v -= period * floor((v - lo) / period);
    atomicOr(status, ST_NAN);
  }
  return v;
}

// block-wide exclusive scan of one int per thread (blockDim.x a multiple of 32);
// returns the exclusive prefix, *total the block's sum
__device__ __forceinline__ int block_excl_scan(int v, int* sh, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = lane < nw ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sh[lane] = t;  // inclusive warp totals
  }
  __syncthreads();
  const int excl = x - v + (w > 0 ? sh[w - 1] : 0);
  *total = sh[nw - 1];
  __syncthreads();
  return excl;
}

// The rebuild worklist (one block): the flagged systems in increasing order with
// the exclusive prefix sums of their slot and cell counts.
// The systems to rebuild: those flagged, and those whose table row (tab, row; tab may
// be null) sets gamma back, which the set-back kernel flags after this list is made.
__global__ void __launch_bounds__(1024) k_rb_worklist(Dev d, const StepScalars* __restrict__ tab,
                                                       int row) {
  __shared__ int sh[32];
  int ba = 0, bb = 0, bc = 0;  // running totals (identical in every thread)
  for (int s0 = 0; s0 < d.nsys; s0 += blockDim.x) {
    const int s = s0 + threadIdx.x;
    const bool f = s < d.nsys && (d.flags[s] != 0 || (tab && tab[row * d.nsys + s].setback));
    int ta, tb, tc;
    const int ea = block_excl_scan(f ? 1 : 0, sh, &ta);
    const int eb = block_excl_scan(f ? d.geom[s].n : 0, sh, &tb);
    const int ec = block_excl_scan(f ? d.geom[s].cols * d.geom[s].rows : 0, sh, &tc);
    if (f) {
      d.work[ba + ea] = s;
      d.woff[ba + ea] = bb + eb;
      d.wcoff[ba + ea] = bc + ec;
    }
    ba += ta;
    bb += tb;
    bc += tc;
  }
  if (threadIdx.x == 0) {
    d.nwork[0] = ba;
    d.nwork[1] = bb;
    d.nwork[2] = bc;
    d.woff[ba] = bb;
    d.wcoff[ba] = bc;
  }
}

__global__ void k_rb_zero(Dev d) {
  if (*d.any == 0) return;
  for_listed_cells(d, [&](int c, int) { d.cell_count[c] = 0; });
}

// find_cells, spherocyl_box.cpp:270-301: wrap, then hash.
//
// A displacement-triggered rebuild happens in the reference inside the corrector
// loop, at the first particle i* whose accumulated displacement exceeds pad/2:
// particles up to i* are wrapped after their update, the others before it, and
// the displacement counters of the latter restart from this step's move.  The
// reference wraps with the box length of the loop (before a resize shrinks it).
// Reproducing that matters under resize, where the reference's predictor pass
// uses the pre-resize box for the minimum image and so depends on which image a
// particle sits at.  Forced rebuilds and set-back steps wrap every particle.
__global__ void k_rb_hash(Dev d, const StepScalars* __restrict__ tab, int row, int mixed) {
  if (*d.any == 0) return;
  for_listed_slots(d, [&](int i, int s) {
    const SysGeom& g = d.geom[s];
    const StepScalars& ts = tab[row * d.nsys + s];
    // pure shear rebuilds after the box update (pure_strain_step_2p,
    // src/cuda/2point_dynamics.cu:2255-2282), so it wraps with the new box
    const double Lx = ts.mode == 3 ? ts.Lx_p : ts.Lx_c, Ly = ts.mode == 3 ? ts.Ly_p : ts.Ly_c;
    double2 p = d.xy[i];
    double phi = d.ph[i];
    double2 mv = make_double2(0.0, 0.0);
    const int istar = d.istar[s];
    if (!mixed && istar != kNoTrigger && !ts.setback && ts.mode != 3 && d.id[i] > istar) {
      double2 p0 = d.s_xy[i];
      p0.x = wrap_bounded(p0.x, 0.0, Lx, Lx, d.status);
      p0.y = wrap_bounded(p0.y, 0.0, Ly, Ly, d.status);
      double ph0 = wrap_bounded(d.s_ph[i], -kRefPi, kRefPi, 2 * kRefPi, d.status);
      p = make_double2(p0.x + d.v0x[i], p0.y + d.v0y[i]);
      phi = ph0 + d.v0p[i];
      if (ts.mode == 1) {
        p.x *= ts.scale;
        p.y *= ts.scale;
      } else if (ts.mode == 2) {
        p.x /= ts.scale;
        p.y /= ts.scale;
      }
      mv = make_double2(p.x - p0.x, p.y - p0.y);
    } else {
      p.x = wrap_bounded(p.x, 0.0, Lx, Lx, d.status);
      p.y = wrap_bounded(p.y, 0.0, Ly, Ly, d.status);
      phi = wrap_bounded(phi, -kRefPi, kRefPi, 2 * kRefPi, d.status);
    }
    d.xy[i] = p;
    d.ph[i] = phi;
    d.nxy_t[i] = mv;  // displacement counter to carry into the new slot
    // the FP64 form divides as the reference does (find_cells); the mixed form,
    // whose records are relative to whatever cell it is given, takes the FP32
    // quotient (two FP64 divisions per particle dominate this kernel on GB300; a
    // particle a rounding error outside its cell is still well inside the 3x3 block
    // its list search covers, whose cells are 0.24 (R + A) wider than the reach)
    int col, rw;
    if (mixed) {
      col = (int)__fdividef((float)p.x, ts.f_Wp);
      rw = (int)__fdividef((float)p.y, ts.f_Hp);
    } else {
      col = (int)(p.x / ts.W_p);
      rw = (int)(p.y / ts.H_p);
    }
    // a coordinate at (or, after a resize, just past) the box edge stays on the grid
    if (col >= g.cols) col = g.cols - 1;
    if (rw >= g.rows) rw = g.rows - 1;
    if (col < 0) col = 0;
    if (rw < 0) rw = 0;
    int c = g.c0 + cell_local(g, col, rw);
    d.cell_tmp[i] = c;
    // one atomic per cell among the converged lanes: the slots arrive in cell order,
    // so neighbouring lanes mostly share a cell (the order inside a cell is settled
    // by k_rb_cellsort)
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, c);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&d.cell_count[c], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    d.rank[i] = base + __popc(peers & ((1u << lane) - 1u));
  });
}

__device__ __forceinline__ int block_sum_int(int v, int* sh) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  if (w == 0) {
    v = lane < nw ? sh[lane] : 0;
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;  // valid in thread 0
}

__global__ void k_rb_chunksum(Dev d) {
  if (*d.any == 0) return;
  int ch = blockIdx.x;
  if (d.flags[d.chunk_sys[ch]] == 0) return;
  __shared__ int sh[32];
  int c0 = d.chunk_c0[ch], nc = d.chunk_nc[ch];
  int v = 0;
  for (int k = threadIdx.x; k < nc; k += blockDim.x) v += d.cell_count[c0 + k];
  v = block_sum_int(v, sh);
  if (threadIdx.x == 0) d.chunk_sum[ch] = v;
}

// One block per system: exclusive scan of its chunk sums (a large system owns a few
// hundred chunks).
__global__ void __launch_bounds__(256) k_rb_sysscan(Dev d) {
  if (*d.any == 0) return;
  const int s = blockIdx.x;
  if (d.flags[s] == 0) return;
  __shared__ int sh[32];
  const SysGeom& g = d.geom[s];
  int off = 0;  // running total (the same in every thread)
  for (int k0 = 0; k0 < g.nchunks; k0 += blockDim.x) {
    const int k = k0 + threadIdx.x;
    const int v = k < g.nchunks ? d.chunk_sum[g.chunk0 + k] : 0;
    int tot;
    const int ex = block_excl_scan(v, sh, &tot);
    if (k < g.nchunks) d.chunk_off[g.chunk0 + k] = off + ex;
    off += tot;
  }
  if (threadIdx.x == 0 && off != g.n) atomicOr(d.status, ST_CELL_OVERFLOW);
}

// One 1024-thread block per chunk: exclusive scan of cell counts.
__global__ void __launch_bounds__(1024) k_rb_cellscan(Dev d) {
  if (*d.any == 0) return;
  int ch = blockIdx.x;
  int s = d.chunk_sys[ch];
  if (d.flags[s] == 0) return;
  __shared__ int warp_tot[32];
  int c0 = d.chunk_c0[ch], nc = d.chunk_nc[ch];
  int k = threadIdx.x;
  int v = k < nc ? d.cell_count[c0 + k] : 0;
  int lane = k & 31, w = k >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;  // inclusive
  }
  __syncthreads();
  int excl = x - v + (w > 0 ? warp_tot[w - 1] : 0);
  if (k < nc) d.cell_start[c0 + k] = d.geom[s].p0 + d.chunk_off[ch] + excl;
}

__global__ void k_rb_scatter(Dev d) {
  if (*d.any == 0) return;
  for_listed_slots(d, [&](int i, int) { d.perm[d.cell_start[d.cell_tmp[i]] + d.rank[i]] = i; });
}

// Order each cell's slots by particle index: the reference's cell lists are
// filled in particle order (spherocyl_box.cpp:277-298).
__global__ void k_rb_cellsort(Dev d) {
  if (*d.any == 0) return;
  for_listed_cells(d, [&](int c, int) {
    int st = d.cell_start[c], n = d.cell_count[c];
    if (n <= 1) return;
    int* P = d.perm + st;
    if (n <= kMaxCellSort) {
      int key[kMaxCellSort], val[kMaxCellSort];
      for (int k = 0; k < n; k++) {
        val[k] = P[k];
        key[k] = d.id[val[k]];
      }
      for (int k = 1; k < n; k++) {
        int kk = key[k], vv = val[k], m = k - 1;
        while (m >= 0 && key[m] > kk) {
          key[m + 1] = key[m];
          val[m + 1] = val[m];
          m--;
        }
        key[m + 1] = kk;
        val[m + 1] = vv;
      }
      for (int k = 0; k < n; k++) P[k] = val[k];
    } else {
      for (int k = 1; k < n; k++) {
        int vv = P[k], kk = d.id[vv], m = k - 1;
        while (m >= 0 && d.id[P[m]] > kk) {
          P[m + 1] = P[m];
          m--;
        }
        P[m + 1] = vv;
      }
    }
  });
}

__global__ void k_rb_gather(Dev d) {
  if (*d.any == 0) return;
  for_listed_slots(d, [&](int i, int) {
    int src = d.perm[i];
    d.s_xy[i] = d.xy[src];
    d.s_ph[i] = d.ph[src];
    d.s_ra[i] = d.ra[src];
    d.s_irc[i] = d.irc[src];
    d.s_id[i] = d.id[src];
    d.s_cell[i] = d.cell_tmp[src];
    double2 mv = d.nxy_t[src];
    d.v0x[i] = mv.x;
    d.v0y[i] = mv.y;
    if (d.fvx) {  // minimiser velocities travel with their particles (predictor copy is dead here)
      d.xy_t[i] = make_double2(d.fvx[src], d.fvy[src]);
      d.ph_t[i] = d.fvp[src];
    }
    if (d.cg0x) {  // and the minimiser's previous forces (stress partials are dead here)
      d.se_part[i] = d.cg0x[src];
      d.se_part[(size_t)d.ntot + i] = d.cg0y[src];
      d.se_part[2 * (size_t)d.ntot + i] = d.cg0p[src];
    }
  });
}

__global__ void k_rb_commit(Dev d, const StepScalars* __restrict__ tab, int row, int mixed) {
  if (*d.any == 0) return;
  for_listed_slots(d, [&](int i, int) {
    double2 p = d.s_xy[i];
    double phi = d.s_ph[i];
    double2 ra = d.s_ra[i];
    d.xy[i] = p;
    d.ph[i] = phi;
    d.ra[i] = ra;
    d.irc[i] = d.s_irc[i];
    d.id[i] = d.s_id[i];
    d.cell[i] = d.s_cell[i];
    d.moved[i] = make_double2(d.v0x[i], d.v0y[i]);
    if (d.fvx) {
      double2 v = d.xy_t[i];
      d.fvx[i] = v.x;
      d.fvy[i] = v.y;
      d.fvp[i] = d.ph_t[i];
    }
    if (d.cg0x) {
      d.cg0x[i] = d.se_part[i];
      d.cg0y[i] = d.se_part[(size_t)d.ntot + i];
      d.cg0p[i] = d.se_part[2 * (size_t)d.ntot + i];
    }
    if (!mixed) {
      double sn, cs;
      sincos(phi, &sn, &cs);
      d.nxy[i] = make_double2(ra.y * cs, ra.y * sn);
    }
  });
}

__global__ void k_rb_clear(Dev d) {
  if (*d.any == 0) return;
  for (int s = threadIdx.x; s < d.nsys; s += blockDim.x) {
    d.flags[s] = 0;
    d.istar[s] = kNoTrigger;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *d.any = 0;
    d.status[1] += 1;  // rebuild chains executed
  }
}

__global__ void k_force_all(Dev d) {
  for (int s = threadIdx.x; s < d.nsys; s += blockDim.x) d.flags[s] = 2;
  if (threadIdx.x == 0) *d.any = 1;
}

// set_back_gamma, spherocyl_box.cpp:524-545 (positions; gamma itself is advanced
// on the host), for the systems whose table row says so.
__device__ __forceinline__ void setback_slot(const Dev& d, const StepScalars* __restrict__ tab,
                                             int row, int i, int s) {
  const StepScalars& ts = tab[row * d.nsys + s];
  if (!ts.setback) return;
  double Lx = ts.Lx_p, Ly = ts.Ly_p;
  double2 p = d.xy[i];
  if (p.y < 0)
    p.y += Ly;
  else if (p.y > Ly)
    p.y -= Ly;
  p.x += (Lx / Ly) * p.y;  // x + y in a square box (Lx / Ly == 1 exactly)
  if (p.x < 0)
    p.x += Lx;
  else
    p.x = wrap_bounded(p.x, -1.0, Lx, Lx, d.status);  // only the "> Lx" loop applies
  d.xy[i] = p;
  if (i == d.geom[s].p0) {
    atomicOr(&d.flags[s], 2);
    atomicExch(d.any, 1);
  }
}

__global__ void k_setback(Dev d, const StepScalars* __restrict__ tab, int row) {
  for_listed_slots(d, [&](int i, int s) { setback_slot(d, tab, row, i, s); });
}

// Recompute the shaft vectors of the FP64 form from the state, e.g. after the
// host replaced positions.
__global__ void k_refresh(Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  double phi = d.ph[i];
  double2 ra = d.ra[i];
  double sn, cs;
  sincos(phi, &sn, &cs);
  d.nxy[i] = make_double2(ra.y * cs, ra.y * sn);
}

// gradient_relax_step, src/cpp/relaxation_dynamics.cpp:11-31
__global__ void k_gd_update(Dev d, const StepScalars* __restrict__ tab, int row) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  int s = d.psys[i];
  const SysGeom& g = d.geom[s];
  const double step = tab[row * d.nsys + s].step;
  if (step == 0.0) return;
  double ddx = step * d.fx[i];
  double ddy = step * d.fy[i];
  double ddp = step * d.tau[i] / d.irc[i].x;
  const double2 p0 = d.xy[i];
  const double phi0 = d.ph[i];
  double2 p = make_double2(p0.x + ddx, p0.y + ddy);
  double phi = phi0 + ddp;
  d.xy[i] = p;
  d.ph[i] = phi;
  d.s_xy[i] = p0;
  d.s_ph[i] = phi0;
  d.v0x[i] = ddx;
  d.v0y[i] = ddy;
  d.v0p[i] = ddp;
  double2 m = d.moved[i];
  m.x += ddx;
  m.y += ddy;
  d.moved[i] = m;
  double2 ra = d.ra[i];
  double sn, cs;
  sincos(phi, &sn, &cs);
  d.nxy[i] = make_double2(ra.y * cs, ra.y * sn);
  if (!(isfinite(p.x) && isfinite(p.y) && isfinite(phi))) atomicOr(d.status, ST_NAN);
  // the reference tests and rebuilds inside the update loop
  if (m.x > 0.5 * g.pad || m.x < -0.5 * g.pad || m.y > 0.5 * g.pad || m.y < -0.5 * g.pad) {
    if (d.flags[s] == 0) atomicOr(&d.flags[s], 1);
    atomicMin(&d.istar[s], d.id[i]);
    if (*d.any == 0) atomicExch(d.any, 1);
  }
}

// Stress/energy: deterministic two-level reduction of the per-slot contributions.
__global__ void k_se_chunk(Dev d) {
  int ch = blockIdx.x;
  int p0 = d.pchunk_p0[ch], np = d.pchunk_np[ch];
  __shared__ double sh[5][32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int comp = 0; comp < 5; comp++) {
    const double* src = d.se_part + (size_t)comp * d.ntot + p0;
    double v = 0.0;
    for (int k = threadIdx.x; k < np; k += blockDim.x) v += src[k];
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[comp][w] = v;
  }
  __syncthreads();
  if (w < 5) {
    double v = lane < nw ? sh[w][lane] : 0.0;
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) d.se_chunk[(size_t)w * d.npchunks + ch] = v;
  }
}

// One block per system: each thread sums its strided share of the system's chunk
// partials in order, then a fixed tree over the block (deterministic).
__global__ void __launch_bounds__(256) k_se_sys(Dev d) {
  const int s = blockIdx.x;
  const SysGeom& g = d.geom[s];
  const int ch0 = g.pch0, ch1 = g.pch0 + pchunk_count(g);
  __shared__ double sh[5][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int comp = 0; comp < 5; comp++) {
    double v = 0.0;
    for (int ch = ch0 + threadIdx.x; ch < ch1; ch += blockDim.x)
      v += d.se_chunk[(size_t)comp * d.npchunks + ch];
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[comp][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double v = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) v += sh[threadIdx.x][k];
    d.se_sys[(size_t)threadIdx.x * d.nsys + s] = v;
  }
}

// se_sys is [5][nsys]; a record is [nsys][5]
__global__ void k_se_store(Dev d, double* dst) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.nsys) return;
  for (int k = 0; k < 5; k++) dst[5 * s + k] = d.se_sys[(size_t)k * d.nsys + s];
}

// set_particle's wrap loop (src/cpp/spherocyl_box.cpp:204-215) for the input state:
// the reference's repeated subtraction, finished by a floor for a value more than
// 64 periods out (where the loop would take that long; not an error here).
__device__ __forceinline__ double wrap_input(double v, double lo, double hi, double period) {
  int it = 0;
  while (v > hi && it < 64) {
    v -= period;
    it++;
  }
  while (v < lo && it < 64) {
    v += period;
    it++;
  }
  if (it >= 64) v -= period * floor((v - lo) / period);
  return v;
}

// Per-particle state of a new handle (set_particle, src/cpp/spherocyl_box.cpp:188-221):
// the wrapped position and angle, (R, A), the moment of inertia I and the rotation
// coefficient RC in the reference's operation order, the particle index and system
// of each slot.  x..A are the caller's arrays: host memory that the GPU reads in
// place where it can address pageable memory, else a device copy.  sys_p0 holds the
// first slot of each system and ntot at [nsys]; sys_L the (Lx, Ly) pairs.
__global__ void k_ingest(Dev d, const double* __restrict__ x, const double* __restrict__ y,
                         const double* __restrict__ phi, const double* __restrict__ R,
                         const double* __restrict__ A, const int* __restrict__ sys_p0,
                         const double* __restrict__ sys_L, int* __restrict__ psys) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.ntot; i += stride) {
    int lo = 0, hi = d.nsys - 1;  // the system whose slot range holds i
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sys_p0[mid] <= i)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int s = lo;
    const double Lx = sys_L[2 * s], Ly = sys_L[2 * s + 1];
    const double r = R[i], a = A[i];
    const double al = a / r;
    const double C = (3 * kRefPi + 24 * al + 6 * kRefPi * al * al + 8 * al * al * al);
    const double area = r * (kRefPi * r + 4 * a);
    d.irc[i] = make_double2(r * r * r * r * C / (6 * area),
                            (8 * al + 6 * kRefPi * al * al + 8 * al * al * al) / C);
    d.ra[i] = make_double2(r, a);
    d.xy[i] = make_double2(wrap_input(x[i], 0.0, Lx, Lx), wrap_input(y[i], 0.0, Ly, Ly));
    d.ph[i] = wrap_input(phi[i], -kRefPi, kRefPi, 2 * kRefPi);
    d.id[i] = i - sys_p0[s];
    psys[i] = s;
  }
}

// Output in the caller's particle order: slot i holds particle p0 + id[i] of its
// system, so each value goes to out[k * ntot + p0 + id[i]].
__global__ void k_unsort_state(Dev d, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const size_t o = (size_t)d.geom[d.psys[i]].p0 + d.id[i];
  const double2 p = d.xy[i];
  out[o] = p.x;
  out[(size_t)d.ntot + o] = p.y;
  out[(size_t)2 * d.ntot + o] = d.ph[i];
}

__global__ void k_unsort_forces(Dev d, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const size_t o = (size_t)d.geom[d.psys[i]].p0 + d.id[i];
  out[o] = d.fx[i];
  out[(size_t)d.ntot + o] = d.fy[i];
  out[(size_t)2 * d.ntot + o] = d.tau[i];
}

inline int nblk(int n, int b) { return (n + b - 1) / b; }

}  // namespace

void launch_rb_worklist(const Dev& d, const StepScalars* tab, int row, cudaStream_t st) {
  k_rb_worklist<<<1, 1024, 0, st>>>(d, tab, row);
}

void launch_rebuild(const Dev& d, bool mixed, const StepScalars* tab, int row, cudaStream_t st,
                    bool listed) {
  const int B = 256;
  // the slot and cell kernels walk the worklist with a fixed grid
  if (!listed) k_rb_worklist<<<1, 1024, 0, st>>>(d, tab, row);
  k_rb_zero<<<kWalkBlocks, B, 0, st>>>(d);
  k_rb_hash<<<kWalkBlocks, B, 0, st>>>(d, tab, row, mixed ? 1 : 0);
  k_rb_chunksum<<<d.nchunks, 256, 0, st>>>(d);
  k_rb_sysscan<<<d.nsys, 256, 0, st>>>(d);
  k_rb_cellscan<<<d.nchunks, 1024, 0, st>>>(d);
  k_rb_scatter<<<kWalkBlocks, B, 0, st>>>(d);
  k_rb_cellsort<<<2 * kWalkBlocks, 128, 0, st>>>(d);
  k_rb_gather<<<kWalkBlocks, B, 0, st>>>(d);
  k_rb_commit<<<kWalkBlocks, B, 0, st>>>(d, tab, row, mixed ? 1 : 0);
  if (mixed) {
    launch_mx_local(d, tab, row, false, st);
    if (d.pass_kind == 1) {
      launch_mx_build_list(d, tab, row, false, st);
      launch_tile_lists(d, false, st);
    } else {
      launch_mx_build_order(d, tab, row, false, st);
    }
  } else {
    launch_build_nbrs(d, tab, row, st);
  }
  k_rb_clear<<<1, 256, 0, st>>>(d);
}

void launch_force_rebuild_all(const Dev& d, cudaStream_t st) { k_force_all<<<1, 256, 0, st>>>(d); }

void launch_clear_flags(const Dev& d, cudaStream_t st) { k_rb_clear<<<1, 256, 0, st>>>(d); }

// Inside a captured FIRE iteration: mark the systems that set back gamma at this row
// and switch the graph's conditional rebuild body on when any system needs a
// rebuild.  (The captured shear steps switch theirs from the corrector pass.)
__global__ void k_pre_rebuild(Dev d, const StepScalars* __restrict__ tab, int row,
                              cudaGraphConditionalHandle cond) {
  __shared__ int need;
  if (threadIdx.x == 0) need = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < d.nsys; s += blockDim.x)
    if (tab[row * d.nsys + s].setback) {
      d.flags[s] |= 2;
      need = 1;
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (need) *d.any = 1;
    cudaGraphSetConditional(cond, (need || *d.any) ? 1u : 0u);
  }
}

void launch_pre_rebuild(const Dev& d, const StepScalars* tab, int row,
                        cudaGraphConditionalHandle cond, cudaStream_t st) {
  k_pre_rebuild<<<1, 256, 0, st>>>(d, tab, row, cond);
}

void launch_setback(const Dev& d, const StepScalars* tab, int row, cudaStream_t st) {
  k_setback<<<kWalkBlocks, 256, 0, st>>>(d, tab, row);
}

void launch_refresh_geometry(const Dev& d, bool mixed, const StepScalars* tab, int row,
                             cudaStream_t st) {
  if (mixed)
    launch_mx_local(d, tab, row, true, st);
  else
    k_refresh<<<nblk(d.ntot, 256), 256, 0, st>>>(d);
}

void launch_gd_update(const Dev& d, bool mixed, const StepScalars* tab, int row, cudaStream_t st) {
  (void)mixed;  // the CPU-compatible gradient descent is a plain FP64 protocol
  k_gd_update<<<nblk(d.ntot, 256), 256, 0, st>>>(d, tab, row);
}

void launch_ingest(const Dev& d, const double* x, const double* y, const double* phi,
                   const double* R, const double* A, const int* sys_p0, const double* sys_L,
                   int* psys, cudaStream_t st) {
  const int blocks = nblk(d.ntot, 256) < 152 * 8 ? nblk(d.ntot, 256) : 152 * 8;
  k_ingest<<<blocks, 256, 0, st>>>(d, x, y, phi, R, A, sys_p0, sys_L, psys);
}

void launch_unsort_state(const Dev& d, double* out, cudaStream_t st) {
  k_unsort_state<<<nblk(d.ntot, 256), 256, 0, st>>>(d, out);
}

void launch_unsort_forces(const Dev& d, double* out, cudaStream_t st) {
  k_unsort_forces<<<nblk(d.ntot, 256), 256, 0, st>>>(d, out);
}

void launch_se_store(const Dev& d, double* dst, cudaStream_t st) {
  k_se_store<<<nblk(d.nsys, 128), 128, 0, st>>>(d, dst);
}

void launch_se_reduce(const Dev& d, cudaStream_t st) {
  k_se_chunk<<<d.npchunks, 256, 0, st>>>(d);
  k_se_sys<<<d.nsys, 256, 0, st>>>(d);
}

}  // namespace sc
