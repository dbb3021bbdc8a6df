// spherocyl_configmaker -- zero-energy random starting configurations, no GPU needed.
//
// Arguments of src/cuda/main_configmaker.cpp:63-103: output directory, N, number of
// configurations, packing fraction, aspect ratio A/R (R1 = 0.5), bidispersity R2/R1.
// As get_0e_configs (src/cuda/spherocyl_box.cpp:1415-1421) with the configuration
// {random, angles in [-pi/2, pi/2], no overlap}, configuration i is placed
// contact-free with seed SC_SEED + i (the reference seeds with time(0) + i) and
// written to sd%010d.dat with i as the time, in the src/cuda layout (strain rate
// 1e-3 and step 1, the box's defaults).
#include <chrono>
#include <cstdio>
#include <vector>

#include "cli_common.hpp"

int main(int argc, char** argv) {
  cli::Args a{argc, argv};
  std::string dir = a.s("Output data directory");
  int n = a.i("Number of particles");
  int configs = a.i("Number of configurations");
  double phi = a.f("Packing Fraction");
  double aspect = a.f("Aspect ratio (i.e. A/R or 2A/D)");
  double bidisp = a.f("Bidispersity ratio: (1 for monodisperse)");
  if (n <= 0 || configs < 0 || !(phi > 0)) {
    std::cerr << "need N > 0, a non-negative number of configurations and a packing > 0"
              << std::endl;
    return 1;
  }
  auto start = std::chrono::steady_clock::now();
  sc_gen_options o;
  sc_default_gen_options(&o);
  o.layout = SC_LAYOUT_RANDOM;
  o.angle_mode = SC_ANGLE_RANDOM;
  o.angle_min = 0.0;  // u in [0, 1]: angles pi u - pi/2 in [-pi/2, pi/2]
  o.angle_max = 1.0;
  o.max_overlap = 0.0;  // zero energy
  const int seed0 = cli::env_int("SC_SEED", 0);
  std::vector<double> x(n), y(n), p(n), R(n), A(n);
  for (int i = 0; i < configs; i++) {
    double L = 0;
    int rc = sc_generate_config(&o, n, phi, aspect, 0.5, bidisp, (uint64_t)(seed0 + i), x.data(),
                                y.data(), p.data(), R.data(), A.data(), &L);
    if (rc) return cli::fail("packing", rc);
    const double hdr[7] = {L, L, phi, 0.0, 0.0, 1e-3, 1.0};
    char name[32];
    snprintf(name, sizeof name, "/sd%010d.dat", i);
    rc = sc_write_positions((dir + name).c_str(), SC_FMT_SD, n, hdr, x.data(), y.data(), p.data(),
                            R.data(), A.data());
    if (rc) return cli::fail("write", rc);
  }
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  std::cout << "\nRun Time: " << secs << std::endl;
  return 0;
}
