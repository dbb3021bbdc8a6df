// sc_pass_mixed.cu -- the mixed-precision form: cell-tile force passes.
//
// Pair geometry and forces in FP32, positions/orientations and the Heun update in
// FP64, stress and energy accumulated in FP64.  No neighbour list is stored: each
// thread takes one particle slot (slots are sorted by cell) and scans the 3x3 block
// of cells around its own cell, whose particles are contiguous slot ranges.  The
// rebuild rule is the reference's (a rebuild when a particle's accumulated
// displacement exceeds pad/2 in x or y, tmarschall/spherocyls
// src/cpp/strain_dynamics.cpp:220-225), and the cell size is the reference's
// (src/cpp/spherocyl_box.cpp:228-232), which bounds every possible contact to the
// 3x3 block, so the set of interacting pairs is exactly the reference's.
//
// A pair is computed with the lower particle index as the reference's "p" from
// both sides, so both threads produce the same FP32 contribution and Newton's
// third law holds exactly pair by pair.
#include "sc_internal.hpp"
#include "sc_pair.cuh"
#include "sc_rec.cuh"

namespace sc {

namespace {

__device__ __forceinline__ void flag_moved(const Dev& d, int s, double2 m, double pad) {
  if (m.x > 0.5 * pad || m.x < -0.5 * pad || m.y > 0.5 * pad || m.y < -0.5 * pad) {
    if (d.flags[s] == 0) atomicOr(&d.flags[s], 1);
    if (*d.any == 0) atomicExch(d.any, 1);
  }
}

template <int MODE, bool SE>
__global__ void __launch_bounds__(256) k_pass_mixed(Dev d, const StepScalars* __restrict__ tab,
                                                   int row) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ntot) return;
  constexpr bool kPred = (MODE == PASS_CORR_STRAIN || MODE == PASS_CORR_RESIZE);
  const int s = d.psys[i];
  const SysGeom& g = d.geom[s];
  const StepScalars& ts = tab[row * d.nsys + s];
  const float4* __restrict__ REC = kPred ? d.rec_t : d.rec;
  const double Wd = kPred ? ts.W_c : ts.W_p;
  const double Hd = kPred ? ts.H_c : ts.H_p;
  const float W = (float)Wd, H = (float)Hd;
  const float gam = (float)(kPred ? ts.gamma_c : ts.gamma_p);
  const bool virial = d.stress_mode == STRESS_VIRIAL;

  const float4 ri = REC[i];
  const float2 rai = d.raf[i];
  const int idi = d.id[i];
  const int lc = d.cell[i] - g.c0;
  const int col = lc % g.cols, rw = lc / g.cols;
  const int ncx = g.cols < 3 ? g.cols : 3, ncy = g.rows < 3 ? g.rows : 3;
  const bool smallx = ncx < 3, smally = ncy < 3;
  const float Lxf = W * g.cols, Lyf = H * g.rows;

  float fx = 0.f, fy = 0.f, tq = 0.f;
  double e_acc = 0.0, pxx = 0.0, pyy = 0.0, pxy = 0.0, pyx = 0.0;

  for (int a = 0; a < ncy; a++) {
    int dr = smally ? a - rw : a - 1;  // small grids: absolute row a
    int r2 = smally ? a : wrap_index(rw + dr, g.rows);
    float oy = -(float)dr * H;
    for (int b = 0; b < ncx; b++) {
      int dc = smallx ? b - col : b - 1;
      int c2 = smallx ? b : wrap_index(col + dc, g.cols);
      float ox = -(float)dc * W;
      int cc = g.c0 + r2 * g.cols + c2;
      int st = d.cell_start[cc];
      int en = st + d.cell_count[cc];
      for (int j = st; j < en; j++) {
        if (j == i) continue;
        float4 rj = REC[j];
        float dx = (ri.x - rj.x) + ox;
        float dy = (ri.y - rj.y) + oy;
        if (smallx) dx += Lxf * (float)((dx < -0.5f * Lxf) - (dx > 0.5f * Lxf));
        if (smally) dy += Lyf * (float)((dy < -0.5f * Lyf) - (dy > 0.5f * Lyf));
        // quick reject: centres farther apart than R+A+R+A (sheared frame bound)
        float2 raj = d.raf[j];
        float reach = rai.x + rai.y + raj.x + raj.y;
        float dxl = fmaf(gam, dy, dx);
        if (dxl * dxl + dy * dy >= reach * reach) continue;
        int idj = d.id[j];
        bool ip = idi < idj;
        PairF32 o;
        bool hit;
        if (ip)
          hit = pair_fp32<SE>(dx, dy, ri.z, ri.w, rai.y, rj.z, rj.w, raj.y, rai.x + raj.x, gam,
                              virial, o);
        else
          hit = pair_fp32<false>(-dx, -dy, rj.z, rj.w, raj.y, ri.z, ri.w, rai.y, raj.x + rai.x,
                                 gam, virial, o);
        if (!hit) continue;
        if (ip) {
          fx += o.fx;
          fy += o.fy;
          tq += o.tp;
          if (SE) {
            e_acc += (double)(o.ov * o.ov);
            if (!virial) {
              pxx += (double)(o.fx * o.cxa) - (double)(o.fx * o.cxb) - (double)(o.fy * o.cxb);
              pyy += (double)(o.fy * o.cya) - (double)(o.fy * o.cyb);
              pxy += (double)(o.fy * o.cxa);
              pyx += (double)(o.fx * o.cya) - (double)(o.fx * o.cyb);
            } else {
              pxx += (double)(o.fx * o.cxa) - (double)(o.fx * o.cxb);
              pyy += (double)(o.fy * o.cya) - (double)(o.fy * o.cyb);
              pxy += (double)(o.fy * o.cxa) - (double)(o.fy * o.cxb);
              pyx += (double)(o.fx * o.cya) - (double)(o.fx * o.cyb);
            }
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
    const double Lx = kPred ? ts.Lx_c : ts.Lx_p, Ly = kPred ? ts.Ly_c : ts.Ly_p;
    const double inv_area = 1.0 / (Lx * Ly);
    d.se_part[i] = e_acc * 0.5 * g.inv_n;
    d.se_part[(size_t)d.ntot + i] = pxx * inv_area;
    d.se_part[(size_t)2 * d.ntot + i] = pyy * inv_area;
    d.se_part[(size_t)3 * d.ntot + i] = pxy * inv_area;
    d.se_part[(size_t)4 * d.ntot + i] = pyx * inv_area;
  }

  const double2 irc = d.irc[i];
  const double dt = ts.step;
  const double Fx = fx, Fy = fy, T = tq;
  const double A = rai.y;
  if (MODE == PASS_FORCE) {
    d.fx[i] = Fx;
    d.fy[i] = Fy;
    d.tau[i] = T;
  } else if (MODE == PASS_PRED_STRAIN || MODE == PASS_PRED_RESIZE) {
    d.fx[i] = Fx;
    d.fy[i] = Fy;
    d.tau[i] = T;
    double phi = d.ph[i];
    double v0x, v0y, v0p;
    if (MODE == PASS_PRED_STRAIN) {
      const double gamma = ts.gamma_p;
      v0x = Fx - gamma * Fy;
      v0y = Fy;
      float iso = 0.5f * (1.f - (float)irc.y * cosf(2.f * (float)phi));
      v0p = T / irc.x - ts.rate * (double)iso;
    } else {
      v0x = Fx;
      v0y = Fy;
      v0p = T / irc.x;
    }
    d.v0x[i] = v0x;
    d.v0y[i] = v0y;
    d.v0p[i] = v0p;
    double2 p = d.xy[i];
    double2 pt = make_double2(p.x + dt * v0x, p.y + dt * v0y);
    double pht = phi + dt * v0p;
    if (MODE == PASS_PRED_RESIZE) {
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
    // the next consumer of the predictor record is the corrector pass of the next
    // step, whose box is the one after this step
    d.rec_t[i] = make_rec(pt, pht, A, col, rw, ts.W_p, ts.H_p);
  } else {
    double pht = d.ph_t[i];
    double ddx, ddy, ddp;
    if (MODE == PASS_CORR_STRAIN) {
      const double gamma = ts.gamma_c;
      double v1x = Fx - gamma * Fy;
      double v1y = Fy;
      float iso = 0.5f * (1.f - (float)irc.y * cosf(2.f * (float)pht));
      double v1p = T / irc.x - ts.rate * (double)iso;
      ddx = 0.5 * dt * (d.v0x[i] + v1x);
      ddy = 0.5 * dt * (d.v0y[i] + v1y);
      ddp = 0.5 * dt * (d.v0p[i] + v1p);
    } else {
      ddx = 0.5 * dt * (d.v0x[i] + Fx);
      ddy = 0.5 * dt * (d.v0y[i] + Fy);
      ddp = 0.5 * dt * (d.v0p[i] + T / irc.x);
    }
    double2 p0 = d.xy[i];
    double2 p = make_double2(p0.x + ddx, p0.y + ddy);
    double phi = d.ph[i] + ddp;
    if (MODE == PASS_CORR_RESIZE) {
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
    double2 m = d.moved[i];
    m.x += p.x - p0.x;
    m.y += p.y - p0.y;
    d.moved[i] = m;
    d.rec[i] = make_rec(p, phi, A, col, rw, ts.W_p, ts.H_p);
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(phi))) atomicOr(d.status, ST_NAN);
    flag_moved(d, s, m, g.pad);
  }
}

template <int MODE, bool SE>
void launch_one(const Dev& d, const StepScalars* tab, int row, cudaStream_t st, int block) {
  int grid = (d.ntot + block - 1) / block;
  k_pass_mixed<MODE, SE><<<grid, block, 0, st>>>(d, tab, row);
}

}  // namespace

void launch_pass_mixed(const Dev& d, int mode, bool se, const StepScalars* tab, int row,
                       cudaStream_t st, int block) {
  if (block <= 0) block = 128;
  switch (mode) {
    case PASS_FORCE:
      se ? launch_one<PASS_FORCE, true>(d, tab, row, st, block)
         : launch_one<PASS_FORCE, false>(d, tab, row, st, block);
      break;
    case PASS_CORR_STRAIN: launch_one<PASS_CORR_STRAIN, false>(d, tab, row, st, block); break;
    case PASS_PRED_STRAIN:
      se ? launch_one<PASS_PRED_STRAIN, true>(d, tab, row, st, block)
         : launch_one<PASS_PRED_STRAIN, false>(d, tab, row, st, block);
      break;
    case PASS_CORR_RESIZE: launch_one<PASS_CORR_RESIZE, false>(d, tab, row, st, block); break;
    case PASS_PRED_RESIZE:
      se ? launch_one<PASS_PRED_RESIZE, true>(d, tab, row, st, block)
         : launch_one<PASS_PRED_RESIZE, false>(d, tab, row, st, block);
      break;
  }
}

}  // namespace sc
