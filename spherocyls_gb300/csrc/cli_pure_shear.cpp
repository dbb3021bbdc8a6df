// spherocyl_pure_shear -- pure-shear run (x stretched, y compressed) on the GPU.
//
// Arguments in the order of the src/cuda pure-shear driver
// (src/cuda/main_pure_shear.cpp:61-150): data file or "r", output directory, N,
// strain rate, step, stop aspect Lx/Ly, position save interval (strain), stress save
// interval (strain), cell padding, shear-direction change (1: rotate the box by
// gamma first, with the total strain reset), and for "r": packing fraction, aspect
// ratio A/R (R1 = 0.5), bidispersity R2/R1, then optionally the initial
// configuration code (0-9) and the aspect-ratio spread (see cli::random_start).  A
// random start fills a box of aspect 1/stop_aspect (main_pure_shear.cpp:168-170).
// SC_PRECISION=mixed selects the mixed form, SC_OUTPUT_FORMAT=sp the src/cpp file
// layout (the default here is the src/cuda one), SC_SEED the seed of the random
// configuration, SC_CONTACTS=2 the two-point contact model of the src/cuda 2p code.
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
  double stop = a.f("Strain stop (Box Aspect Lx/Ly)");
  double pos_save = a.f("Position data save rate");
  double se_save = a.f("Stress data save rate");
  double pad = a.f("Cell padding");
  int flip = a.i("Change shear direction (1 to rotate)");
  if (!(stop > 0)) {
    std::cerr << "the stop aspect must be positive" << std::endl;
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
                               A.data(), &L, 1.0 / stop, &Ly);
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
  if (flip == 1) {
    // main_pure_shear.cpp:261-265
    if ((rc = sc_set_total_gamma(h, -1, 0.0)) || (rc = sc_rotate_shear(h, -1)))
      return cli::fail("shear direction", rc, h);
  }
  unsigned long t_end = 0;
  rc = sc_run_pure_strain(h, dir.c_str(), stop, pos_save, se_save, t0, cli::out_format(SC_FMT_SD),
                          &t_end);
  if (rc) return cli::fail("run", rc, h);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  std::cout << "\nRun Time: " << secs << std::endl;
  sc_destroy(h);
  return 0;
}
