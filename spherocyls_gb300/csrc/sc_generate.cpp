// sc_generate.cpp -- seeded, crossing-free random packings (host code).
//
// The reference places particles with rand()/time(0) and rejects only touching
// or crossing placements (random_configuration, tmarschall/spherocyls
// src/cpp/spherocyl_box.cpp:694-790, check_particle_cross :597-645).  Uniform
// random centres at packing fractions near 0.85 put crossing spines into the
// initial state, and a crossing pair gives a 0/0 force direction in the pair
// routine (src/cpp/strain_dynamics.cpp:58-62) that turns the run to NaN within
// tens of steps.  This generator is reproducible (SplitMix64 stream per seed) and
// rejects a placement while its spine comes closer than min_sep * (R_i + R_j) to
// an earlier spine, under periodic minimum-image distances.
//
// sc_generate_config adds the reference's other initial configurations
// (place_spherocyls, place_random_0e_spherocyls, place_spherocyl_grid, set_shapes:
// src/cuda/spherocyl_box.cpp:1063-1394): zero-energy placement, grid placement with
// random row offsets, random / evenly spaced / aligned angles, optionally drawn
// from the isolated-rotation steady-shear distribution (uniformToAngleDist,
// :1044-1061), and gamma-distributed aspect ratios, all from one seeded stream.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/spherocyl.h"
#include "sc_segments.hpp"

namespace {

using sc_seg::seg_seg;

struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// standard normal (Box-Muller)
double normal(SplitMix64& r) {
  double u1 = r.uniform(), u2 = r.uniform();
  if (u1 < 1e-300) u1 = 1e-300;
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

// Gamma(k, 1) by Marsaglia and Tsang, ACM TOMS 26, 363 (2000); k < 1 through
// Gamma(k + 1) * U^(1/k).
double gamma_k(SplitMix64& r, double k) {
  if (k < 1.0) {
    double u = r.uniform();
    if (u < 1e-300) u = 1e-300;
    return gamma_k(r, k + 1.0) * std::pow(u, 1.0 / k);
  }
  const double d = k - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
  for (;;) {
    double z, v;
    do {
      z = normal(r);
      v = 1.0 + c * z;
    } while (v <= 0);
    v = v * v * v;
    double u = r.uniform();
    if (u < 1.0 - 0.0331 * z * z * z * z) return d * v;
    if (u > 0 && std::log(u) < 0.5 * z * z + d * (1.0 - v + std::log(v))) return d * v;
  }
}

// uniformToAngleDist (src/cuda/spherocyl_box.cpp:1044-1061): u in [0, 1] to an
// angle in [-pi/2, pi/2); with `shear` the steady-shear distribution of an
// isolated particle with rotation coefficient C.
double angle_of(double u, double C, bool shear) {
  const double pi = 3.14159265358979323846;
  if (!shear || C == 0) return pi * u - pi / 2;
  return std::atan(std::sqrt(1 - C * C) * std::tan(pi * (u - 0.5)) / (1 + C));
}

}  // namespace

extern "C" void sc_default_gen_options(sc_gen_options* o) {
  if (!o) return;
  o->layout = SC_LAYOUT_RANDOM;
  o->angle_mode = SC_ANGLE_RANDOM;
  o->angle_min = 0.0;
  o->angle_max = 1.0;
  o->shear_angles = 0;
  o->min_sep = 0.1;
  o->max_overlap = -1.0;
  o->a_sigma = 0.0;
}

// box_aspect = Lx/Ly; the area Lx*Ly is the square box's L^2
// (the pure-shear driver's start box, src/cuda/main_pure_shear.cpp:168-170)
extern "C" int sc_generate_config_rect(const sc_gen_options* opt, int n, double packing,
                                       double a_over_r, double r_small, double r_ratio,
                                       double box_aspect, uint64_t seed, double* x, double* y,
                                       double* phi, double* R, double* A, double* Lx_out,
                                       double* Ly_out) {
  sc_gen_options o;
  if (opt)
    o = *opt;
  else
    sc_default_gen_options(&o);
  if (n < 2 || !(packing > 0 && packing < 1) || !(a_over_r >= 0) || !(r_small > 0) ||
      !(r_ratio > 0) || !(o.min_sep >= 0) || !(o.a_sigma >= 0) ||
      !(o.angle_min >= 0 && o.angle_max <= 1 && o.angle_min <= o.angle_max) ||
      (o.layout != SC_LAYOUT_RANDOM && o.layout != SC_LAYOUT_GRID) ||
      (o.angle_mode != SC_ANGLE_RANDOM && o.angle_mode != SC_ANGLE_EVEN) || !(o.max_overlap < 1) ||
      !(box_aspect > 0 && box_aspect < 1e6 && 1.0 / box_aspect < 1e6) || !x || !y || !phi ||
      !R || !A || !Lx_out || !Ly_out)
    return SC_E_ARG;
  const double pi = 3.14159265358979323846;
  SplitMix64 rng{seed * 0x2545F4914F6CDD1Dull + 0x9876543ull};
  // shapes (set_shapes): species alternate by index; a/R fixed or Gamma with mean
  // a_over_r and standard deviation a_sigma * a_over_r
  double filled = 0.0, rmax = 0.0, amax = 0.0;
  const double k = o.a_sigma > 0 ? 1.0 / (o.a_sigma * o.a_sigma) : 0.0;
  for (int i = 0; i < n; i++) {
    R[i] = (i % 2 == 0) ? r_small : r_small * r_ratio;
    double alpha = a_over_r;
    if (o.a_sigma > 0 && a_over_r > 0) alpha = gamma_k(rng, k) * a_over_r / k;
    A[i] = alpha * R[i];
    filled += pi * R[i] * R[i] + 4.0 * A[i] * R[i];
    rmax = std::fmax(rmax, R[i]);
    amax = std::fmax(amax, A[i]);
  }
  const double L = std::sqrt(filled / packing);
  const double Lx = L * std::sqrt(box_aspect), Ly = L / std::sqrt(box_aspect);
  *Lx_out = Lx;
  *Ly_out = Ly;
  // rotation coefficient of the largest shape (place_spherocyls' dC)
  const double al = rmax > 0 ? amax / rmax : 0.0;
  const double C = al * (8 + 6 * pi * al + 8 * al * al) /
                   (3 * pi + 24 * al + 6 * pi * al * al + 8 * al * al * al);
  // rejection: spine distance below min_sep * sigma, or (max_overlap >= 0) below
  // sqrt(1 - max_overlap) * sigma (check_for_crosses / check_for_contacts)
  const double sep = o.max_overlap >= 0 ? std::fmax(o.min_sep, std::sqrt(1.0 - o.max_overlap))
                                        : o.min_sep;
  const double reach = 2.0 * amax + 2.0 * sep * rmax;
  int ngx = (int)(Lx / std::fmax(reach, 1e-300)), ngy = (int)(Ly / std::fmax(reach, 1e-300));
  if (ngx > 2048) ngx = 2048;
  if (ngy > 2048) ngy = 2048;
  const bool gridded = ngx >= 3 && ngy >= 3;
  if (!gridded) ngx = ngy = 1;
  const double gwx = Lx / ngx, gwy = Ly / ngy;
  std::vector<std::vector<int>> grid((size_t)ngx * ngy);
  // grid layout (place_spherocyl_grid): cells of W x H, one particle each, rows
  // shifted by a random offset of up to +-(R + A)
  int ncols = 1, nrows = 1;
  double W = Lx, H = Ly;
  std::vector<double> row_off;
  if (o.layout == SC_LAYOUT_GRID) {
    const double aspect = (amax + rmax) / rmax;
    ncols = std::max(1, (int)std::sqrt(n / aspect * box_aspect));
    nrows = (n + ncols - 1) / ncols;
    W = Lx / ncols;
    H = Ly / nrows;
    if (W < 2 * (amax + rmax) || H < 2 * rmax) return SC_E_ARG;  // does not fit
    row_off.assign(nrows, 0.0);
    for (int r = 1; r < nrows; r++) row_off[r] = (rmax + amax) * (1.0 - 2.0 * rng.uniform());
  }
  const long max_tries = 1000000;
  for (int i = 0; i < n; i++) {
    long tries = 0;
    for (;;) {
      if (++tries > max_tries) return SC_E_NOCONV;
      double xi, yi;
      if (o.layout == SC_LAYOUT_GRID) {
        const int r = i / ncols, c = i % ncols;
        xi = c * W + (amax + rmax) + row_off[r] + (W - 2 * (amax + rmax)) * rng.uniform();
        yi = r * H + rmax + (H - 2 * rmax) * rng.uniform();
        xi -= Lx * std::floor(xi / Lx);
        yi -= Ly * std::floor(yi / Ly);
      } else {
        xi = Lx * rng.uniform();
        yi = Ly * rng.uniform();
      }
      double u;
      if (o.angle_mode == SC_ANGLE_EVEN)
        u = o.angle_min + (2.0 * i + 1.0) * (o.angle_max - o.angle_min) / (2.0 * n);
      else
        u = o.angle_min + (o.angle_max - o.angle_min) * rng.uniform();
      const double pi_ = angle_of(u, C, o.shear_angles != 0);
      double ux = A[i] * std::cos(pi_), uy = A[i] * std::sin(pi_);
      int gx = gridded ? std::min((int)(xi / gwx), ngx - 1) : 0;
      int gy = gridded ? std::min((int)(yi / gwy), ngy - 1) : 0;
      bool ok = true;
      int span = gridded ? 1 : 0;
      for (int a = -span; a <= span && ok; a++)
        for (int b = -span; b <= span && ok; b++) {
          int cx = (gx + b + ngx) % ngx, cy = (gy + a + ngy) % ngy;
          for (int j : grid[(size_t)cy * ngx + cx]) {
            double dx = xi - x[j], dy = yi - y[j];
            dx -= Lx * std::round(dx / Lx);
            dy -= Ly * std::round(dy / Ly);
            double vx = A[j] * std::cos(phi[j]), vy = A[j] * std::sin(phi[j]);
            double dd = seg_seg(dx, dy, ux, uy, 0.0, 0.0, vx, vy);
            if (dd < sep * (R[i] + R[j])) {
              ok = false;
              break;
            }
          }
        }
      if (!ok) continue;
      x[i] = xi;
      y[i] = yi;
      phi[i] = pi_;
      grid[(size_t)gy * ngx + gx].push_back(i);
      break;
    }
  }
  return SC_OK;
}

extern "C" int sc_generate_config(const sc_gen_options* opt, int n, double packing,
                                  double a_over_r, double r_small, double r_ratio, uint64_t seed,
                                  double* x, double* y, double* phi, double* R, double* A,
                                  double* L_out) {
  double Ly = 0;
  return sc_generate_config_rect(opt, n, packing, a_over_r, r_small, r_ratio, 1.0, seed, x, y,
                                 phi, R, A, L_out, &Ly);
}

extern "C" int sc_generate_packing(int n, double packing, double a_over_r, double r_small,
                                   double r_ratio, uint64_t seed, double min_sep, double* x,
                                   double* y, double* phi, double* R, double* A, double* L_out) {
  if (n < 2 || !(packing > 0 && packing < 1) || !(a_over_r >= 0) || !(r_small > 0) ||
      !(r_ratio > 0) || !(min_sep >= 0) || !x || !y || !phi || !R || !A || !L_out)
    return SC_E_ARG;
  const double pi = 3.14159265358979323846;
  double filled = 0.0, rmax = 0.0, amax = 0.0;
  for (int i = 0; i < n; i++) {
    R[i] = (i % 2 == 0) ? r_small : r_small * r_ratio;
    A[i] = a_over_r * R[i];
    filled += pi * R[i] * R[i] + 4.0 * A[i] * R[i];
    rmax = std::fmax(rmax, R[i]);
    amax = std::fmax(amax, A[i]);
  }
  const double L = std::sqrt(filled / packing);
  *L_out = L;
  // any two spines closer than min_sep*(Ri+Rj) have centres within reach
  const double reach = 2.0 * amax + 2.0 * min_sep * rmax;
  int ng = (int)(L / std::fmax(reach, 1e-300));
  if (ng > 2048) ng = 2048;
  const bool gridded = ng >= 3;
  if (!gridded) ng = 1;
  const double gw = L / ng;
  std::vector<std::vector<int>> grid((size_t)ng * ng);
  SplitMix64 rng{seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
  const long max_tries = 1000000;
  for (int i = 0; i < n; i++) {
    long tries = 0;
    for (;;) {
      if (++tries > max_tries) return SC_E_NOCONV;
      double xi = L * rng.uniform(), yi = L * rng.uniform(), pi_ = pi * rng.uniform();
      double ux = A[i] * std::cos(pi_), uy = A[i] * std::sin(pi_);
      int gx = gridded ? std::min((int)(xi / gw), ng - 1) : 0;
      int gy = gridded ? std::min((int)(yi / gw), ng - 1) : 0;
      bool ok = true;
      int span = gridded ? 1 : 0;
      for (int a = -span; a <= span && ok; a++)
        for (int b = -span; b <= span && ok; b++) {
          int cx = (gx + b + ng) % ng, cy = (gy + a + ng) % ng;
          for (int j : grid[(size_t)cy * ng + cx]) {
            double dx = xi - x[j], dy = yi - y[j];
            dx -= L * std::round(dx / L);
            dy -= L * std::round(dy / L);
            double vx = A[j] * std::cos(phi[j]), vy = A[j] * std::sin(phi[j]);
            double dd = seg_seg(dx, dy, ux, uy, 0.0, 0.0, vx, vy);
            if (dd < min_sep * (R[i] + R[j])) {
              ok = false;
              break;
            }
          }
        }
      if (!ok) continue;
      x[i] = xi;
      y[i] = yi;
      phi[i] = pi_;
      grid[(size_t)gy * ng + gx].push_back(i);
      break;
    }
  }
  return SC_OK;
}
