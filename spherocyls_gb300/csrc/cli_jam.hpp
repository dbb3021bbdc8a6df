// The find-jam and y-compression drivers (src/cuda/main_2point_findjam.cpp:63-261,
// src/cuda/main_2point_ycompress.cpp, the same arguments with a target energy):
// data file or "r", output directory, N, resize step (the drivers' "resize rate",
// the first relative length step), integration step, energy at jamming / target
// energy (per unit area, calc_fe_2p's normalisation), position and stress save
// rates (read and, as there, not used by the bisection), cell padding, and for "r":
// packing fraction, aspect ratio A/R (R1 = 0.5), bidispersity R2/R1, then optionally
// the initial configuration code (0-9) and the aspect-ratio spread (see
// cli::random_start).  Contacts are the two-point model of the src/cuda 2p code
// unless SC_CONTACTS=1 (the one-point rule of the src/cuda 1p find-jam driver,
// main_1point_findjam.cpp); each resize relaxes with the conjugate gradient in the
// default FP64 form (SC_PRECISION=mixed: FIRE); SC_SEED seeds the random
// configuration.  Files: sd_stress_energy.dat, sd%010d.dat per resize, the final
// state as sd%010d.bin.
#pragma once
#include <chrono>
#include <cstdio>
#include <vector>

#include "cli_common.hpp"

namespace cli {

// y_only: the y-compression driver (target energy prompt, sc_run_y_compress)
inline int jam_main(int argc, char** argv, bool y_only) {
  cli::Args a{argc, argv};
  std::string file = a.s("Data file ('r' for random)");
  std::string dir = a.s("Output data directory");
  int n = a.i("Number of particles");
  double step = a.f("Resize rate (epsilon)");
  double dt = a.f("Integration step size");
  double e_jam = a.f(y_only ? "Target Energy" : "Energy at jamming");
  (void)a.f("Position data save rate");
  (void)a.f("Stress data save rate");
  double pad = a.f("Cell padding");
  if (!(step != 0) || !(e_jam > 0)) {
    std::cerr << "need a non-zero resize step and a positive jamming energy" << std::endl;
    return 1;
  }
  std::vector<double> x, y, p, R, A;
  double L = 0, Ly = 0, gamma = 0, gamma_total = 0;
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
  }
  auto start = std::chrono::steady_clock::now();
  sc_options opt;
  sc_default_options(&opt);
  opt.precision = cli::precision();
  opt.contact_model = cli::env_int("SC_CONTACTS", 2) == 1 ? SC_CONTACT_ONE : SC_CONTACT_TWO;
  sc_handle* h = nullptr;
  if (Ly == 0) Ly = L;
  int rc = sc_create_rect(&opt, 1, &n, &L, &Ly, &pad, x.data(), y.data(), p.data(), R.data(),
                          A.data(), &h);
  if (rc) return cli::fail("create", rc);
  if ((rc = sc_set_step(h, -1, dt)) || (rc = sc_set_gamma(h, -1, gamma)) ||
      (rc = sc_set_total_gamma(h, -1, gamma_total)))
    return cli::fail("setup", rc, h);
  int steps = 0;
  double phi = 0;
  // both take the magnitude of the step (resize_to_energy_2p, y_resize_to_energy_2p)
  const double mag = step < 0 ? -step : step;
  rc = y_only ? sc_run_y_compress(h, dir.c_str(), e_jam, mag, 1e-13, 200000, &steps, &phi)
              : sc_run_find_jam(h, dir.c_str(), e_jam, mag, 1e-13, 200000, &steps, &phi);
  if (rc) return cli::fail(y_only ? "y compress" : "find jam", rc, h);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  std::printf("\nResizes: %d\nPacking fraction: %.10f\nRun Time: %g\n", steps, phi, secs);
  sc_destroy(h);
  return 0;
}

}  // namespace cli
