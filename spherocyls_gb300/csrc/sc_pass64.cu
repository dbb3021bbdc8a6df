// sc_pass64.cu -- the plain FP64 form: neighbour-list build and force passes.
//
// Compiled with -fmad=false: together with the operation order of sc_pair.cuh and
// the explicit Heun arithmetic below, every pair contribution and every position
// update is the reference's own sequence of IEEE operations
// (tmarschall/spherocyls src/cpp/strain_dynamics.cpp:17-235,
// src/cpp/resize_dynamics.cpp:164-243, src/cpp/spherocyl_box.cpp:303-355).
//
// One thread per particle slot gathers over the particle's full neighbour list
// (column-major, one coalesced index load per entry) and computes each pair with
// the lower particle index as the reference's "p", so the two threads that visit a
// pair compute bit-identical contributions.  The epilogue fuses the Heun
// predictor or corrector for the slot.
#include "sc_internal.hpp"
#include "sc_pair.cuh"

namespace sc {

namespace {

// check_neighbors, src/cpp/spherocyl_box.cpp:303-318, with p the lower index.
__device__ __forceinline__ bool nbr_criterion(double2 pp, double2 pq, double sig, double pad,
                                              double gamma, double Lx, double Ly) {
  double dY = pp.y - pq.y;
  dY += Ly * (double)((dY < -0.5 * Ly) - (dY > 0.5 * Ly));
  if (fabs(dY) < sig + pad) {
    double dX = pp.x - pq.x;
    dX += Lx * (double)((dX < -0.5 * Lx) - (dX > 0.5 * Lx));
    double dXmax = dX + 0.5 * dY;  // dX at the largest gamma of the list lifetime
    dX += gamma * dY;
    if (fabs(dX) < sig + pad || fabs(dXmax) < sig + pad) return true;
  }
  return false;
}

__global__ void __launch_bounds__(128) k_build_nbrs(Dev d, const StepScalars* __restrict__ tab,
                                                   int row) {
  if (*d.any == 0) return;
  for_listed_slots(d, [&](int i, int s) {
    const SysGeom g = d.geom[s];
    const StepScalars ts = tab[row * d.nsys + s];
    double2 pi = d.xy[i];
    double2 rai = d.ra[i];
    int idi = d.id[i];
    int c = d.cell[i] - g.c0;
    int col, rw;
    cell_colrow(g, c, &col, &rw);
    // 3x3 block of cells; a dimension with fewer than three cells is scanned once
    // per distinct cell (the reference would list such cells twice).
    int ncx = g.cols < 3 ? g.cols : 3, ncy = g.rows < 3 ? g.rows : 3;
    int cnt = 0;
    for (int a = 0; a < ncy; a++) {
      int r2 = ncy == 3 ? wrap_index(rw + a - 1, g.rows) : a;
      for (int b = 0; b < ncx; b++) {
        int c2 = ncx == 3 ? wrap_index(col + b - 1, g.cols) : b;
        int cc = g.c0 + cell_local(g, c2, r2);
        int st = d.cell_start[cc], nn = d.cell_count[cc];
        for (int j = st; j < st + nn; j++) {
          if (j == i) continue;
          int idj = d.id[j];
          double2 pj = d.xy[j];
          double2 raj = d.ra[j];
          bool ip = idi < idj;
          // S = R_p + A_p + R_q + A_q summed in the reference's order
          double sig = ip ? rai.x + rai.y + raj.x + raj.y : raj.x + raj.y + rai.x + rai.y;
          bool hit = ip ? nbr_criterion(pi, pj, sig, g.pad, ts.gamma_p, ts.Lx_p, ts.Ly_p)
                        : nbr_criterion(pj, pi, sig, g.pad, ts.gamma_p, ts.Lx_p, ts.Ly_p);
          if (hit) {
            if (cnt < d.maxn) d.nbr[(size_t)cnt * d.ntot + i] = j;
            cnt++;
          }
        }
      }
    }
    d.nbr_n[i] = cnt;
    if (cnt > d.maxn) atomicOr(d.status, ST_NBR_OVERFLOW);
  });
}

// The reference rebuilds inside its corrector loop as soon as particle i has
// moved more than pad/2 (strain_dynamics.cpp:220-225, resize_dynamics.cpp:222-227);
// the lowest such index per system is kept so the rebuild can reproduce which
// particles the reference wrapped before, and which after, their update.
__device__ __forceinline__ void flag_moved(const Dev& d, int s, int id, double2 m, double pad) {
  if (m.x > 0.5 * pad || m.x < -0.5 * pad || m.y > 0.5 * pad || m.y < -0.5 * pad) {
    atomicMin(&d.istar[s], id);
    request_rebuild(d, s);
  }
}

// The FP64 pass of one slot: its pairs over its full list, then the Heun epilogue.
template <int MODE, bool SE, bool TWO, bool FAST = false>
__device__ __forceinline__ void pass64_slot(const Dev& d, const StepScalars* __restrict__ tab,
                                            int row, int i) {
  constexpr bool kPred =
      (MODE == PASS_CORR_STRAIN || MODE == PASS_CORR_RESIZE || MODE == PASS_ENERGY_T);
  int s = d.psys[i];
  if (d.skip && d.skip[s]) return;  // a converged minimiser system
  const SysGeom& g = d.geom[s];
  const StepScalars ts = tab[row * d.nsys + s];
  const double2* __restrict__ XY = kPred ? d.xy_t : d.xy;
  const double2* __restrict__ NXY = kPred ? d.nxy_t : d.nxy;
  const double gamma = kPred ? ts.gamma_c : ts.gamma_p;
  const double Lx = kPred ? ts.Lx_c : ts.Lx_p;
  const double Ly = kPred ? ts.Ly_c : ts.Ly_p;
  const bool virial = d.stress_mode == STRESS_VIRIAL;
  constexpr bool two_point = TWO;
  const double two_n = 2.0 * g.n;

  double2 pi = XY[i];
  double2 ni = NXY[i];
  double2 rai = d.ra[i];
  int idi = d.id[i];
  double fx = 0.0, fy = 0.0, tq = 0.0;
  double se0 = 0.0, se1 = 0.0, se2 = 0.0, se3 = 0.0, se4 = 0.0;
  int cnt = d.nbr_n[i];
  if (cnt > d.maxn) cnt = d.maxn;
  const float fpi_x = (float)ni.x, fpi_y = (float)ni.y, fai = (float)rai.y;
  for (int k0 = 0; k0 < cnt; k0 += 64) {
    // FP32 screen of up to 64 entries: the FP64 contact code then runs only for the
    // entries that may touch, in list order, so the sums are unchanged bit for bit
    unsigned long long cand = 0ull;
    const int kend = cnt - k0 < 64 ? cnt : k0 + 64;
    for (int k = k0; k < kend; k++) {
      const int j = d.nbr[(size_t)k * d.ntot + i];
      const double2 pj = XY[j];
      const double2 nj = NXY[j];
      const double2 raj = d.ra[j];
      double dX = pi.x - pj.x, dY = pi.y - pj.y;
      dX += Lx * (double)((dX < -0.5 * Lx) - (dX > 0.5 * Lx));
      dY += Ly * (double)((dY < -0.5 * Ly) - (dY > 0.5 * Ly));
      dX += gamma * dY;
      if (may_touch_fp32((float)dX, (float)dY, fpi_x, fpi_y, fai, (float)nj.x, (float)nj.y,
                         (float)raj.y, (float)(rai.x + raj.x)))
        cand |= 1ull << (k - k0);
    }
    while (cand) {
      const int k = k0 + __ffsll((long long)cand) - 1;
      cand &= cand - 1ull;
      int j = d.nbr[(size_t)k * d.ntot + i];
      double2 pj = XY[j];
      double2 nj = NXY[j];
      double2 raj = d.ra[j];
      int idj = d.id[j];
      // the lower particle index plays the reference's "p": select the operands (one
      // copy of the pair code per warp) rather than branch into two
      const bool ip = idi < idj;
      const double2 pP = ip ? pi : pj, pQ = ip ? pj : pi;
      const double2 nP = ip ? ni : nj, nQ = ip ? nj : ni;
      const double2 rP = ip ? rai : raj, rQ = ip ? raj : rai;
      PairF64 o;
      const bool hit =
          two_point ? pair2_fp64<SE, FAST>(pP.x - pQ.x, pP.y - pQ.y, nP.x, nP.y, rP.y, nQ.x,
                                           nQ.y, rQ.y, rP.x + rQ.x, gamma, Lx, Ly, two_n, o)
                    : pair_fp64<SE, FAST>(pP.x - pQ.x, pP.y - pQ.y, nP.x, nP.y, rP.y, nQ.x, nQ.y,
                                          rQ.y, rP.x + rQ.x, gamma, Lx, Ly, virial, two_n, o);
      if (hit) {
        if (ip) {
          fx += o.fx;
          fy += o.fy;
          tq += o.tp;
          if (SE) {
            se0 += o.e;
            se1 += o.pxx;
            se2 += o.pyy;
            se3 += o.pxy;
            se4 += o.pyx;
          }
        } else {
          fx -= o.fx;
          fy -= o.fy;
          tq += o.tq;
        }
      }
    }
  }
  if (SE) {
    d.se_part[i] = se0;
    d.se_part[(size_t)d.ntot + i] = se1;
    d.se_part[(size_t)2 * d.ntot + i] = se2;
    d.se_part[(size_t)3 * d.ntot + i] = se3;
    d.se_part[(size_t)4 * d.ntot + i] = se4;
  }

  const double2 irc = d.irc[i];  // (I, RC)
  const double dt = ts.step;
  if (MODE == PASS_FORCE) {
    d.fx[i] = fx;
    d.fy[i] = fy;
    d.tau[i] = tq;
  } else if (MODE == PASS_PRED_STRAIN) {
    // strain_step predictor, strain_dynamics.cpp:187-199
    d.fx[i] = fx;
    d.fy[i] = fy;
    d.tau[i] = tq;
    double phi = d.ph[i];
    double v0x = fx - gamma * fy;
    double v0y = fy;
    double v0p = tq / irc.x - ts.rate * iso_rot64(irc.y, phi);
    d.v0x[i] = v0x;
    d.v0y[i] = v0y;
    d.v0p[i] = v0p;
    double2 p = d.xy[i];
    double2 pt = make_double2(p.x + dt * v0x, p.y + dt * v0y);
    double pht = phi + dt * v0p;
    d.xy_t[i] = pt;
    d.ph_t[i] = pht;
    double sn, cs;
    sincos(pht, &sn, &cs);
    d.nxy_t[i] = make_double2(rai.y * cs, rai.y * sn);
  } else if (MODE == PASS_CORR_STRAIN) {
    // strain_step corrector, strain_dynamics.cpp:203-219
    double pht = d.ph_t[i];
    double v1x = fx - gamma * fy;
    double v1y = fy;
    double v1p = tq / irc.x - ts.rate * iso_rot64(irc.y, pht);
    double ddx = 0.5 * dt * (d.v0x[i] + v1x);
    double ddy = 0.5 * dt * (d.v0y[i] + v1y);
    double ddp = 0.5 * dt * (d.v0p[i] + v1p);
    double2 p = d.xy[i];
    const double2 p0 = p;
    const double phi0 = d.ph[i];
    p.x += ddx;
    p.y += ddy;
    double phi = phi0 + ddp;
    d.xy[i] = p;
    d.ph[i] = phi;
    // pre-step state and increments, for a rebuild that follows this step
    d.s_xy[i] = p0;
    d.s_ph[i] = phi0;
    d.v0x[i] = ddx;
    d.v0y[i] = ddy;
    d.v0p[i] = ddp;
    double2 m = d.moved[i];
    m.x += ddx;
    m.y += ddy;
    d.moved[i] = m;
    double sn, cs;
    sincos(phi, &sn, &cs);
    d.nxy[i] = make_double2(rai.y * cs, rai.y * sn);
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(phi))) atomicOr(d.status, ST_NAN);
    flag_moved(d, s, idi, m, g.pad);
  } else if (MODE == PASS_PRED_RESIZE) {
    // resize_step predictor, resize_dynamics.cpp:172-191
    d.fx[i] = fx;
    d.fy[i] = fy;
    d.tau[i] = tq;
    d.v0x[i] = fx;
    d.v0y[i] = fy;
    d.v0p[i] = tq;
    double2 p = d.xy[i];
    double2 pt;
    double pht;
    if (ts.mode == 3) {
      // pure-shear predictor (pure_euler_est_2p, src/cuda/2point_dynamics.cu:1882-1891,
      // with unit drag and the torque over I): the affine flow (+x/2, -y/2) times the
      // strain rate, and the isolated rotation -RC sin(2 phi)/2, by an Euler step
      const double phi = d.ph[i];
      pt = make_double2(p.x + dt * (fx + 0.5 * ts.rate * p.x),
                        p.y + dt * (fy - 0.5 * ts.rate * p.y));
      pht = phi + dt * (tq / irc.x + ts.rate * (-0.5 * irc.y * sin(2 * phi)));
    } else {
      pt = make_double2(p.x + dt * fx, p.y + dt * fy);
      pht = d.ph[i] + dt * tq / irc.x;
      if (ts.mode == 1) {
        pt.x *= ts.scale;
        pt.y *= ts.scale;
      } else if (ts.mode == 2) {
        pt.x /= ts.scale;
        pt.y /= ts.scale;
      }
    }
    d.xy_t[i] = pt;
    d.ph_t[i] = pht;
    double sn, cs;
    sincos(pht, &sn, &cs);
    d.nxy_t[i] = make_double2(rai.y * cs, rai.y * sn);
  } else if (MODE == PASS_CORR_RESIZE) {
    double2 p0 = d.xy[i];
    const double phi0 = d.ph[i];
    double2 p;
    double phi, ddx, ddy, ddp;
    if (ts.mode == 3) {
      // pure-shear corrector (pure_heun_corr_2p, src/cuda/2point_dynamics.cu:2140-2173):
      // the predicted state plus dt/2 times the change of the contact forces
      ddx = 0.5 * dt * (fx - d.v0x[i]);
      ddy = 0.5 * dt * (fy - d.v0y[i]);
      ddp = 0.5 * dt * (tq / irc.x - d.v0p[i] / irc.x);
      const double2 pt = d.xy_t[i];
      p = make_double2(pt.x + ddx, pt.y + ddy);
      phi = d.ph_t[i] + ddp;
    } else {
      // resize_step corrector, resize_dynamics.cpp:194-218
      ddx = 0.5 * dt * (d.v0x[i] + fx);
      ddy = 0.5 * dt * (d.v0y[i] + fy);
      ddp = 0.5 * dt * (d.v0p[i] + tq) / irc.x;
      p = make_double2(p0.x + ddx, p0.y + ddy);
      phi = phi0 + ddp;
      if (ts.mode == 1) {
        p.x *= ts.scale;
        p.y *= ts.scale;
      } else if (ts.mode == 2) {
        p.x /= ts.scale;
        p.y /= ts.scale;
      }
    }
    d.xy[i] = p;
    d.ph[i] = phi;
    d.s_xy[i] = p0;
    d.s_ph[i] = phi0;
    d.v0x[i] = ddx;
    d.v0y[i] = ddy;
    d.v0p[i] = ddp;
    double2 m = d.moved[i];
    m.x += p.x - p0.x;
    m.y += p.y - p0.y;
    d.moved[i] = m;
    double sn, cs;
    sincos(phi, &sn, &cs);
    d.nxy[i] = make_double2(rai.y * cs, rai.y * sn);
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(phi))) atomicOr(d.status, ST_NAN);
    flag_moved(d, s, idi, m, g.pad);
  }
}

template <int MODE, bool SE, bool TWO, bool FAST = false>
__global__ void __launch_bounds__(128) k_pass64(Dev d, const StepScalars* __restrict__ tab,
                                               int row) {
  if (MODE == PASS_CORR_STRAIN || MODE == PASS_CORR_RESIZE) mark_pending_rebuilds(d, tab, row);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  pass64_slot<MODE, SE, TWO, FAST>(d, tab, row, i);
}

// ---- stress and energy of the mixed form, in FP64 ----
//
// The mixed form advances with FP32 pair forces, but the stress tensor and the
// energy it reports are those of the FP64 form at its state: on the steps that
// record them, the compensated state (FP32 value plus FP32 compensation, about
// 48 bits) is widened to FP64 relative to each particle's cell centre, the shaft
// vectors are recomputed in FP64, and every listed pair is evaluated by the FP64
// pair code (the reference's operation order, lower particle index as "p") with
// the sums of calc_se (src/cpp/spherocyl_box.cpp:425-522).  The quantities then
// differ from the FP64 form's only through the states themselves.

// FP64 local positions and shaft vectors of the state (scratch: the FP64 predictor
// arrays, which the mixed form does not use)
__global__ void k_mx_se_prep(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  const float4 r = d.rec[i];
  const float4 c = d.mc[i];
  const double phi = (double)c.z + (double)c.w;
  const double A = d.ra[i].y;
  double sn, cs;
  sincos(phi, &sn, &cs);
  d.xy_t[i] = make_double2((double)r.x + (double)c.x, (double)r.y + (double)c.y);
  d.nxy_t[i] = make_double2(A * cs, A * sn);
}

// The mixed form's FP64 stress and energy of the state, one block per 128 slots.
// Each pair is taken once, from its lower particle index, over the mixed list
// (entries: slot | cell offset code), with the state's scalars (the _p fields).
// Phase 1: each thread marks, in windows of 64 list entries, the entries it owns
// that pass an FP32 screen (a conservative bound on the segment distance, see
// may_touch_fp32).  Phase 2: the block evaluates the marked pairs 128 at a time,
// one per thread whatever the lane owning it, in FP64 with shared reciprocals
// (FAST: this stress is the mixed form's, checked against the FP64 form to 1e-9, not
// the reference's rounding).  Phase 3: each owner adds the results of its own pairs
// in list order.  The sums are those of a per-slot loop over the list, and
// deterministic; the FP64 work runs on full warps instead of the lanes that happen
// to own a touching pair.
constexpr int kSeBlock = 128;

// position of set bit r (0-based, counted from bit 0) of m; m has more than r bits set
__device__ __forceinline__ int nth_set_bit64(unsigned long long m, int r) {
  for (int q = 0; q < r; q++) m &= m - 1ull;
  return __ffsll((long long)m) - 1;
}

template <bool TWO>
__global__ void __launch_bounds__(kSeBlock) k_mx_se64(Dev d, const StepScalars* __restrict__ tab,
                                                     int row) {
  // the owners' particle data and system scalars, for whichever thread evaluates
  // their pairs
  __shared__ double o_px[kSeBlock], o_py[kSeBlock], o_nx[kSeBlock], o_ny[kSeBlock];
  __shared__ double o_R[kSeBlock], o_A[kSeBlock];
  __shared__ double o_W[kSeBlock], o_H[kSeBlock], o_gam[kSeBlock], o_Lx[kSeBlock],
      o_Ly[kSeBlock], o_iLL[kSeBlock], o_2n[kSeBlock], o_i2n[kSeBlock];
  __shared__ unsigned long long mask[kSeBlock];
  __shared__ int off[kSeBlock + 1];
  __shared__ int sh_scan[kSeBlock / 32];
  __shared__ double res[5][kSeBlock];
  const int t = threadIdx.x;
  const int i = blockIdx.x * kSeBlock + t;
  const bool valid = i < d.ntot;
  const bool virial = d.stress_mode == STRESS_VIRIAL;
  int cnt = 0, idi = 0;
  float fnx = 0.f, fny = 0.f, fai = 0.f;
  double px = 0, py = 0, Lx = 1, Ly = 1, gamma = 0, W = 0, H = 0, Ri = 0;
  if (valid) {
    const int s = d.psys[i];
    const SysGeom& g = d.geom[s];
    const StepScalars& ts = tab[row * d.nsys + s];
    W = ts.W_p;
    H = ts.H_p;
    gamma = ts.gamma_p;
    Lx = ts.Lx_p;
    Ly = ts.Ly_p;
    const double2 pi = d.xy_t[i], ni = d.nxy_t[i], rai = d.ra[i];
    px = pi.x;
    py = pi.y;
    Ri = rai.x;
    o_px[t] = pi.x;
    o_py[t] = pi.y;
    o_nx[t] = ni.x;
    o_ny[t] = ni.y;
    o_R[t] = rai.x;
    o_A[t] = rai.y;
    o_W[t] = W;
    o_H[t] = H;
    o_gam[t] = gamma;
    o_Lx[t] = Lx;
    o_Ly[t] = Ly;
    o_iLL[t] = 1.0 / (Lx * Ly);
    o_2n[t] = 2.0 * g.n;
    o_i2n[t] = 0.5 * g.inv_n;
    fnx = (float)ni.x;
    fny = (float)ni.y;
    fai = (float)rai.y;
    idi = d.id[i];
    cnt = min(d.nbr_n[i], d.maxn);
  }
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  // the block's longest list sets the number of 64-entry windows
  int kmax = cnt;
  for (int o = 16; o; o >>= 1) kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
  if ((t & 31) == 0) sh_scan[t >> 5] = kmax;
  __syncthreads();
  kmax = 0;
  for (int w = 0; w < kSeBlock / 32; w++) kmax = max(kmax, sh_scan[w]);
  for (int k0 = 0; k0 < kmax; k0 += 64) {
    // phase 1: this window's owned entries that may touch
    unsigned long long m = 0ull;
    const int kend = min(cnt, k0 + 64);
    for (int k = k0; k < kend; k++) {
      const unsigned e = (unsigned)d.nbr[(size_t)k * d.ntot + i];
      const int j = (int)(e & kSlotMask);
      if (!(idi < d.id[j])) continue;
      const double2 pj = d.xy_t[j];
      const double2 nj = d.nxy_t[j];
      const double Aj = d.ra[j].y, Rj = d.ra[j].x;
      double sx = (px - pj.x) + (double)(1 - (int)((e >> 28) & 3u)) * W;
      double sy = (py - pj.y) + (double)(1 - (int)(e >> 30)) * H;
      sx += Lx * (double)((sx < -0.5 * Lx) - (sx > 0.5 * Lx));
      sy += Ly * (double)((sy < -0.5 * Ly) - (sy > 0.5 * Ly));
      sx += gamma * sy;
      if (may_touch_fp32((float)sx, (float)sy, fnx, fny, fai, (float)nj.x, (float)nj.y,
                         (float)Aj, (float)(Ri + Rj)))
        m |= 1ull << (k - k0);
    }
    mask[t] = m;
    const int c = __popcll(m);
    // exclusive scan of the counts over the block
    int v = c;
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v, o);
      if ((t & 31) >= o) v += u;
    }
    __syncthreads();  // sh_scan is free again
    if ((t & 31) == 31) sh_scan[t >> 5] = v;
    __syncthreads();
    int base_w = 0;
    for (int w = 0; w < (t >> 5); w++) base_w += sh_scan[w];
    off[t] = base_w + v - c;
    int total = 0;
    for (int w = 0; w < kSeBlock / 32; w++) total += sh_scan[w];
    if (t == 0) off[kSeBlock] = total;
    __syncthreads();
    // phases 2 and 3, 128 pairs at a time
    for (int b0 = 0; b0 < total; b0 += kSeBlock) {
      const int p = b0 + t;
      if (p < total) {
        // the owner: the last thread whose offset is at most p
        int lo = 0, hi = kSeBlock - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (off[mid] <= p) lo = mid; else hi = mid - 1;
        }
        const int o = lo;
        const int k = k0 + nth_set_bit64(mask[o], p - off[o]);
        const int io = blockIdx.x * kSeBlock + o;
        const unsigned e = (unsigned)d.nbr[(size_t)k * d.ntot + io];
        const int j = (int)(e & kSlotMask);
        const double2 pj = d.xy_t[j];
        const double2 nj = d.nxy_t[j];
        const double2 raj = d.ra[j];
        const double dX = (o_px[o] - pj.x) + (double)(1 - (int)((e >> 28) & 3u)) * o_W[o];
        const double dY = (o_py[o] - pj.y) + (double)(1 - (int)(e >> 30)) * o_H[o];
        PairF64 r;
        const bool hit =
            TWO ? pair2_fp64<true, true>(dX, dY, o_nx[o], o_ny[o], o_A[o], nj.x, nj.y, raj.y,
                                         o_R[o] + raj.x, o_gam[o], o_Lx[o], o_Ly[o], o_2n[o], r,
                                         o_iLL[o], o_i2n[o])
                : pair_fp64<true, true>(dX, dY, o_nx[o], o_ny[o], o_A[o], nj.x, nj.y, raj.y,
                                        o_R[o] + raj.x, o_gam[o], o_Lx[o], o_Ly[o], virial,
                                        o_2n[o], r, o_iLL[o], o_i2n[o]);
        res[0][t] = hit ? r.e : 0.0;
        res[1][t] = hit ? r.pxx : 0.0;
        res[2][t] = hit ? r.pyy : 0.0;
        res[3][t] = hit ? r.pxy : 0.0;
        res[4][t] = hit ? r.pyx : 0.0;
      }
      __syncthreads();
      // each owner adds its pairs of this batch, in list order (a pair that does
      // not touch adds zeros, as the per-slot loop skipped it)
      const int q0 = max(off[t], b0), q1 = min(off[t] + c, b0 + kSeBlock);
      for (int q = q0; q < q1; q++)
        for (int comp = 0; comp < 5; comp++) acc[comp] += res[comp][q - b0];
      __syncthreads();
    }
  }
  if (valid)
    for (int comp = 0; comp < 5; comp++) d.se_part[(size_t)comp * d.ntot + i] = acc[comp];
}

template <int MODE, bool SE>
void launch_one(const Dev& d, const StepScalars* tab, int row, cudaStream_t st) {
  int block = 128;
  int grid = (d.ntot + block - 1) / block;
  if (d.contact_model == 1)
    k_pass64<MODE, SE, true><<<grid, block, 0, st>>>(d, tab, row);
  else
    k_pass64<MODE, SE, false><<<grid, block, 0, st>>>(d, tab, row);
}

}  // namespace

void launch_pass_fp64(const Dev& d, int mode, bool se, const StepScalars* tab, int row,
                      cudaStream_t st, bool fast) {
  if (fast && mode == PASS_FORCE && !se) {
    // the minimiser's force evaluation (shared reciprocals, see qdiv)
    const int block = 128, grid = (d.ntot + block - 1) / block;
    if (d.contact_model == 1)
      k_pass64<PASS_FORCE, false, true, true><<<grid, block, 0, st>>>(d, tab, row);
    else
      k_pass64<PASS_FORCE, false, false, true><<<grid, block, 0, st>>>(d, tab, row);
    return;
  }
  switch (mode) {
    case PASS_FORCE:
      se ? launch_one<PASS_FORCE, true>(d, tab, row, st) : launch_one<PASS_FORCE, false>(d, tab, row, st);
      break;
    case PASS_CORR_STRAIN: launch_one<PASS_CORR_STRAIN, false>(d, tab, row, st); break;
    case PASS_PRED_STRAIN:
      se ? launch_one<PASS_PRED_STRAIN, true>(d, tab, row, st)
         : launch_one<PASS_PRED_STRAIN, false>(d, tab, row, st);
      break;
    case PASS_CORR_RESIZE: launch_one<PASS_CORR_RESIZE, false>(d, tab, row, st); break;
    case PASS_PRED_RESIZE:
      se ? launch_one<PASS_PRED_RESIZE, true>(d, tab, row, st)
         : launch_one<PASS_PRED_RESIZE, false>(d, tab, row, st);
      break;
    case PASS_ENERGY_T: launch_one<PASS_ENERGY_T, true>(d, tab, row, st); break;
  }
}

void launch_mx_se64(const Dev& d, const StepScalars* tab, int row, cudaStream_t st) {
  const int grid = (d.ntot + kSeBlock - 1) / kSeBlock;
  k_mx_se_prep<<<grid, kSeBlock, 0, st>>>(d);
  if (d.contact_model == 1)
    k_mx_se64<true><<<grid, kSeBlock, 0, st>>>(d, tab, row);
  else
    k_mx_se64<false><<<grid, kSeBlock, 0, st>>>(d, tab, row);
}

void launch_build_nbrs(const Dev& d, const StepScalars* tab, int row, cudaStream_t st) {
  k_build_nbrs<<<2 * kWalkBlocks, 128, 0, st>>>(d, tab, row);
}

}  // namespace sc
