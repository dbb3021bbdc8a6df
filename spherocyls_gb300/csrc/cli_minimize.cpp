// spherocyl_minimize -- fixed-step gradient-descent relaxation to zero energy.
//
// Arguments of src/cpp/main_relax.cpp:63-147: data file or "r", output directory,
// N, step, maximum steps, position save interval (steps), stress save interval
// (steps; read and, as in the reference, not used), cell padding, and for "r":
// packing fraction, half-shaft length A, radius R (monodisperse).
#include <chrono>
#include <vector>

#include "cli_common.hpp"

int main(int argc, char** argv) {
  cli::Args a{argc, argv};
  std::string file = a.s("Data file ('r' for random)");
  std::string dir = a.s("Output data directory");
  int n = a.i("Number of particles");
  double dt = a.f("Integration step size");
  int max_steps = a.i("Maximum relaxation steps (n)");
  int pos_save = a.i("Position data save rate (n)");
  (void)a.i("Stress data save rate (n)");
  double pad = a.f("Cell padding");
  std::vector<double> x, y, p, R, A;
  double L = 0, gamma = 0, gamma_total = 0;
  if (file == "r") {
    double phi = a.f("Packing Fraction");
    double ha = a.f("Half-shaft length");
    double r = a.f("Radius");
    x.resize(n), y.resize(n), p.resize(n), R.resize(n), A.resize(n);
    int rc = sc_generate_packing(n, phi, ha / r, r, 1.0, cli::env_int("SC_SEED", 0), 0.1,
                                 x.data(), y.data(), p.data(), R.data(), A.data(), &L);
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
  }
  auto start = std::chrono::steady_clock::now();
  sc_options opt;
  sc_default_options(&opt);
  sc_handle* h = nullptr;
  int rc = sc_create(&opt, 1, &n, &L, &pad, x.data(), y.data(), p.data(), R.data(), A.data(), &h);
  if (rc) return cli::fail("create", rc);
  if ((rc = sc_set_step(h, -1, dt)) || (rc = sc_set_gamma(h, -1, gamma)) ||
      (rc = sc_set_total_gamma(h, -1, gamma_total)))
    return cli::fail("setup", rc, h);
  int steps = 0;
  rc = sc_run_minimize(h, dir.c_str(), max_steps, 0.0, pos_save, &steps);
  if (rc) return cli::fail("run", rc, h);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  std::cout << (steps < max_steps ? "\nEncountered zero energy" : "\nMaximum relaxation steps reached")
            << "\nRun Time: " << secs << std::endl;
  sc_destroy(h);
  return 0;
}
