// cli_common.hpp -- argument reading shared by the command-line drivers.
//
// The reference's drivers take positional arguments from argv, and prompt for and
// read each missing one from standard input, so that "driver < input_file" works
// with one value per line (src/cpp/main.cpp:20-61, input/input_key.txt:1-5).
#pragma once

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "../../include/spherocyl.h"

namespace cli {

struct Args {
  int argc;
  char** argv;
  int n = 0;
  std::string next(const char* what) {
    ++n;
    if (argc > n) {
      std::cout << what << ": " << argv[n] << std::endl;
      return argv[n];
    }
    std::cout << what << ": " << std::flush;
    std::string v;
    if (!(std::cin >> v)) {
      std::cerr << "\nmissing input: " << what << std::endl;
      std::exit(1);
    }
    return v;
  }
  bool more() const { return argc > n + 1; }
  std::string s(const char* what) { return next(what); }
  int i(const char* what) { return std::atoi(next(what).c_str()); }
  double f(const char* what) { return std::atof(next(what).c_str()); }
};

// Options that have no positional field in the reference: environment variables.
inline int env_int(const char* name, int dflt) {
  const char* v = std::getenv(name);
  return v ? std::atoi(v) : dflt;
}
inline int precision() {
  const char* v = std::getenv("SC_PRECISION");
  return (v && std::string(v) == "mixed") ? SC_PREC_MIXED : SC_PREC_FP64;
}
inline int out_format(int dflt = SC_FMT_SP) {
  const char* v = std::getenv("SC_OUTPUT_FORMAT");
  if (!v) return dflt;
  return std::string(v) == "sd" ? SC_FMT_SD : (std::string(v) == "sp" ? SC_FMT_SP : dflt);
}

// time of a continued run: the last 14 characters of the file name are
// "##########.dat" (src/cpp/main.cpp:154-157)
inline unsigned long time_from_name(std::string f) {
  if (f.size() > 3 && f.compare(f.size() - 3, 3, ".gz") == 0) f.resize(f.size() - 3);
  if (f.size() < 14) return 0;
  return std::strtoul(f.substr(f.size() - 14, 10).c_str(), nullptr, 10);
}

// The optional initial-configuration fields of a random start ('r'): the
// configuration code 0-8 (random / zero-energy / grid positions, each with random,
// evenly spaced or aligned angles) or 9 (type, angle range, allowed overlap, angle
// distribution read explicitly), then the aspect-ratio spread
// (src/cuda/main.cpp:119-149), mapped onto sc_generate_config.  Without the fields
// the start is random with random angles.
// box_aspect = Lx/Ly of the start box (L receives Lx, Ly the height).
inline int random_start(Args& a, int n, double phi, double aspect, double bidisp, double* x,
                        double* y, double* p, double* R, double* A, double* L,
                        double box_aspect = 1.0, double* Ly = nullptr) {
  sc_gen_options o;
  sc_default_gen_options(&o);
  if (a.more()) {
    int config = a.i("Initial configuration (0: random, 1: random-uniform, 2: random-aligned, "
                     "3: zero-energy, 4: zero-energy-uniform, 5: zero-energy-aligned, 6: grid, "
                     "7: grid-uniform, 8: grid-aligned, 9: other-specified)");
    double overlap = 1.0;
    if (config == 9) {
      o.layout = a.i("Position configuration type (0: random, 1: grid)") ? SC_LAYOUT_GRID
                                                                          : SC_LAYOUT_RANDOM;
      o.angle_min = a.f("Minimum angle");
      o.angle_max = a.f("Maximum angle");
      overlap = a.f("Allowed overlap (min 0, max 1)");
      o.angle_mode = a.i("Angle distribution type (0: random, 1: uniform)") ? SC_ANGLE_EVEN
                                                                              : SC_ANGLE_RANDOM;
    } else if (config >= 0 && config < 9) {
      o.layout = config < 6 ? SC_LAYOUT_RANDOM : SC_LAYOUT_GRID;
      o.angle_min = 0.0;
      o.angle_max = config % 3 == 2 ? 0.0 : 1.0;
      overlap = (config >= 3 && config < 6) ? 0.0 : 1.0;
      o.angle_mode = config % 3 == 0 ? SC_ANGLE_RANDOM : SC_ANGLE_EVEN;
    } else {
      std::cerr << "unknown initial configuration " << config << std::endl;
      return SC_E_ARG;
    }
    // overlap >= 1: only crossing spines are rejected
    o.max_overlap = overlap < 1.0 ? overlap : -1.0;
    o.a_sigma = a.f("Aspect ratio distribution width (relative deviation)");
  }
  double ly = 0;
  int rc = sc_generate_config_rect(&o, n, phi, aspect, 0.5, bidisp, box_aspect,
                                   env_int("SC_SEED", 0), x, y, p, R, A, L, &ly);
  if (Ly) *Ly = ly;
  return rc;
}

inline int fail(const char* what, int rc, sc_handle* h = nullptr) {
  std::cerr << what << ": " << sc_status_string(rc) << ": " << sc_last_error(h) << std::endl;
  return 1;
}

}  // namespace cli
