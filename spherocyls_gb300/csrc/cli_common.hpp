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
inline int out_format() {
  const char* v = std::getenv("SC_OUTPUT_FORMAT");
  return (v && std::string(v) == "sd") ? SC_FMT_SD : SC_FMT_SP;
}

// time of a continued run: the last 14 characters of the file name are
// "##########.dat" (src/cpp/main.cpp:154-157)
inline unsigned long time_from_name(const std::string& f) {
  if (f.size() < 14) return 0;
  return std::strtoul(f.substr(f.size() - 14, 10).c_str(), nullptr, 10);
}

inline int fail(const char* what, int rc, sc_handle* h = nullptr) {
  std::cerr << what << ": " << sc_status_string(rc) << ": " << sc_last_error(h) << std::endl;
  return 1;
}

}  // namespace cli
