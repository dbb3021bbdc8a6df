// spherocyl_strain -- Lees-Edwards shear run (new or continued) on the GPU.
//
// Arguments in the order of input/input_key.txt:7-22 (the src/cuda driver's order,
// src/cuda/main.cpp:63-125): data file or "r", output directory, N, strain rate,
// step, run length (strain), position save interval (strain), stress save interval
// (strain), cell padding, shear-direction change (0: none, 1: reverse, 2: rotate, 3:
// shear to a maximum gamma without set-back, then rotate), and for "r": packing
// fraction, aspect ratio A/R (R1 = 0.5), bidispersity R2/R1, then optionally the
// initial configuration code (0-9) and the aspect-ratio spread (see
// cli::random_start); for change 3 the maximum gamma comes last (main.cpp:269-275).
// SC_PRECISION=mixed selects the mixed form, SC_OUTPUT_FORMAT=sd the src/cuda file
// layout, SC_SEED the seed of the random configuration, SC_CONTACTS=2 the two-point
// contact model of the src/cuda 2p code.
#include <chrono>
#include <vector>

#include "cli_common.hpp"

int main(int argc, char** argv) {
  cli::Args a{argc, argv};
  std::string file = a.s("Data file ('r' for random)");
  std::string dir = a.s("Output data directory");
  int n = a.i("Number of particles");
  double rate = a.f("Strain rate");
  double dt = a.f("Integration step size");
  double run = a.f("Strain run length (gamma)");
  double pos_save = a.f("Position data save rate");
  double se_save = a.f("Stress data save rate");
  double pad = a.f("Cell padding");
  int flip = a.i("Change shear direction (1 to reverse, 2 to rotate by gamma, 3 to increase "
                  "gamma and rotate)");
  if (flip < 0 || flip > 3) {
    std::cerr << "shear-direction change must be 0, 1 (reverse), 2 (rotate) or 3" << std::endl;
    return 1;
  }
  std::vector<double> x, y, p, R, A;
  double L = 0, Ly = 0, gamma = 0, gamma_total = 0;
  unsigned long t0 = 0;
  if (file == "r") {
    double phi = a.f("Packing Fraction");
    double aspect = a.f("Aspect ratio (A/R)");
    double bidisp = a.f("Bidispersity ratio (R2/R1)");
    x.resize(n), y.resize(n), p.resize(n), R.resize(n), A.resize(n);
    int rc = cli::random_start(a, n, phi, aspect, bidisp, x.data(), y.data(), p.data(), R.data(),
                               A.data(), &L);
    if (rc) return cli::fail("packing", rc);
  } else {
    int nf = 0;
    double hdr[7];
    int rc = sc_read_positions(file.c_str(), &nf, hdr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (rc) return cli::fail("read", rc);
    if (nf != n) std::cerr << "Warning: Number of particles in data file may not match requested number" << std::endl;
    x.resize(nf), y.resize(nf), p.resize(nf), R.resize(nf), A.resize(nf);
    rc = sc_read_positions(file.c_str(), &nf, hdr, x.data(), y.data(), p.data(), R.data(), A.data());
    if (rc) return cli::fail("read", rc);
    n = nf;
    L = hdr[0];
    Ly = hdr[1];
    gamma = hdr[3];
    gamma_total = hdr[4];
    if (hdr[5] != rate) std::cerr << "Warning: Strain rate in data file does not match the requested rate" << std::endl;
    if (hdr[6] != dt) std::cerr << "Warning: Integration step size in data file does not match requested step" << std::endl;
    t0 = cli::time_from_name(file);
  }
  auto start = std::chrono::steady_clock::now();
  sc_options opt;
  sc_default_options(&opt);
  opt.precision = cli::precision();
  if (cli::env_int("SC_CONTACTS", 1) == 2) opt.contact_model = SC_CONTACT_TWO;
  sc_handle* h = nullptr;
  if (Ly == 0) Ly = L;
  int rc = sc_create_rect(&opt, 1, &n, &L, &Ly, &pad, x.data(), y.data(), p.data(), R.data(),
                          A.data(), &h);
  if (rc) return cli::fail("create", rc);
  if ((rc = sc_set_strain_rate(h, -1, rate)) || (rc = sc_set_step(h, -1, dt)) ||
      (rc = sc_set_gamma(h, -1, gamma)) || (rc = sc_set_total_gamma(h, -1, gamma_total)))
    return cli::fail("setup", rc, h);
  if (flip == 3) {
    // main.cpp:269-275: shear to the maximum gamma first
    double gmax = a.f("Max gamma to shear before rotation");
    long k = 0;
    if ((rc = sc_strain_to_gamma(h, gmax, &k))) return cli::fail("shear to gamma", rc, h);
  }
  if (flip >= 1) {
    // main.cpp:258-275: total strain restarts from zero in the new direction
    if ((rc = sc_set_total_gamma(h, -1, 0.0)) ||
        (rc = flip == 1 ? sc_flip_shear(h, -1) : sc_rotate_shear(h, -1)))
      return cli::fail("shear direction", rc, h);
  }
  unsigned long t_end = 0;
  rc = sc_run_strain(h, dir.c_str(), run, pos_save, se_save, t0, cli::out_format(), &t_end);
  if (rc) return cli::fail("run", rc, h);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  std::cout << "\nRun Time: " << secs << std::endl;
  sc_destroy(h);
  return 0;
}
