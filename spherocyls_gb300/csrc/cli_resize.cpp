// spherocyl_resize -- affine compression or expansion to a target packing fraction.
//
// Arguments as for spherocyl_strain with the substitutions of input/input_key.txt:26-30:
// resize rate instead of strain rate, final packing fraction instead of run length,
// and no shear-direction field; for "r": initial packing fraction, aspect ratio
// A/R (R1 = 0.5), bidispersity R2/R1, optionally the initial configuration code
// (0-9) and the aspect-ratio spread (see cli::random_start).  Position files are
// read with the standard header (the src/cpp resize driver's headerless legacy
// column layout, src/cpp/main_resize.cpp:336-349, is not supported).  SC_CONTACTS=2
// selects the two-point contacts of the src/cuda 2p resize driver
// (src/cuda/main_2point_resize.cpp, resize_box_2p).
#include <chrono>
#include <vector>

#include "cli_common.hpp"

int main(int argc, char** argv) {
  cli::Args a{argc, argv};
  std::string file = a.s("Data file ('r' for random)");
  std::string dir = a.s("Output data directory");
  int n = a.i("Number of particles");
  double rate = a.f("Resize rate");
  double dt = a.f("Integration step size");
  double final_phi = a.f("Final packing fraction");
  double pos_save = a.f("Position data save rate");
  double se_save = a.f("Stress data save rate");
  double pad = a.f("Cell padding");
  std::vector<double> x, y, p, R, A;
  double L = 0, gamma = 0, gamma_total = 0;
  unsigned long t0 = 0;
  if (file == "r") {
    double phi = a.f("Starting Packing Fraction");
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
    x.resize(nf), y.resize(nf), p.resize(nf), R.resize(nf), A.resize(nf);
    rc = sc_read_positions(file.c_str(), &nf, hdr, x.data(), y.data(), p.data(), R.data(), A.data());
    if (rc) return cli::fail("read", rc);
    n = nf;
    L = hdr[0];
    gamma = hdr[3];
    gamma_total = hdr[4];
    t0 = cli::time_from_name(file);
  }
  auto start = std::chrono::steady_clock::now();
  sc_options opt;
  sc_default_options(&opt);
  opt.precision = cli::precision();
  if (cli::env_int("SC_CONTACTS", 1) == 2) opt.contact_model = SC_CONTACT_TWO;
  sc_handle* h = nullptr;
  int rc = sc_create(&opt, 1, &n, &L, &pad, x.data(), y.data(), p.data(), R.data(), A.data(), &h);
  if (rc) return cli::fail("create", rc);
  if ((rc = sc_set_resize_rate(h, -1, rate)) || (rc = sc_set_step(h, -1, dt)) ||
      (rc = sc_set_gamma(h, -1, gamma)) || (rc = sc_set_total_gamma(h, -1, gamma_total)))
    return cli::fail("setup", rc, h);
  unsigned long t_end = 0;
  rc = sc_run_resize(h, dir.c_str(), final_phi, pos_save, se_save, t0, cli::out_format(), &t_end);
  if (rc) return cli::fail("run", rc, h);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  std::cout << "\nRun Time: " << secs << std::endl;
  sc_destroy(h);
  return 0;
}
