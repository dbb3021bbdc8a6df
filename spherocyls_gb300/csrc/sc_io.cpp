// sc_io.cpp -- position files, stress/energy time series and the run protocols that
// write them (host code).
//
// Formats follow tmarschall/spherocyls:
//  * src/cpp position file (save_positions, src/cpp/spherocyl_box.cpp:410-423):
//    header "N L packing gamma gamma_total rate dt", rows "x y phi R A", written by
//    an ostream with precision 14; files sp%010lu.dat.
//  * src/cuda position file (save_positions, src/cuda/strain_dynamics.cu:820-843):
//    header "%d %.17g %.17g %f %.17g %.14g %g %g" (N Lx Ly packing gamma gamma_total
//    rate dt), rows "%.17g %.17g %.17g %.2g %.17g"; files sd%010lu.dat.
//  * stress/energy lines: src/cpp "t E Pxx Pyy Pxy" with the ostream default
//    precision (strain_dynamics.cpp:245,291,298), src/cuda "%lu %.7g x6"
//    (t E Pxx Pyy P Pxy Pyx, strain_dynamics.cu:697).
// The reader is the reference's DatFileInput with a header row
// (src/cpp/file_input.h:24-76): whitespace-separated columns, header length 7
// (one box length) or 8 (Lx, Ly; src/cuda/main.cpp:201), plain or gzip-compressed
// (GzFileInput, src/cpp/gz_file_input.cpp).
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/spherocyl.h"
#include "sc_host.hpp"

namespace {


int io_fail(sc::Handle* h, int code, const std::string& msg) {
  if (h) {
    h->err = msg;
    h->last_status = code;
  } else {
    sc::g_noh_error = msg;
  }
  return code;
}

std::string pos_name(const std::string& dir, const char* prefix, unsigned long t) {
  char buf[32];
  snprintf(buf, sizeof buf, "%s%010lu.dat", prefix, t);
  return dir + "/" + buf;
}

// positions of one system in input order
int system_state(sc_handle* H, int sys, std::vector<double>& x, std::vector<double>& y,
                 std::vector<double>& p) {
  sc::Handle& h = H->h;
  std::vector<double> X(h.ntot), Y(h.ntot), P(h.ntot);
  int rc = sc_get_state(H, X.data(), Y.data(), P.data());
  if (rc) return rc;
  const sc::HostSys& S = h.hs[sys];
  x.assign(X.begin() + S.p0, X.begin() + S.p0 + S.n);
  y.assign(Y.begin() + S.p0, Y.begin() + S.p0 + S.n);
  p.assign(P.begin() + S.p0, P.begin() + S.p0 + S.n);
  return SC_OK;
}

// One stress/energy record in the chosen layout.
void se_line(std::ostream& o, int format, unsigned long t, const double* se, bool resize,
             double packing) {
  if (format == SC_FMT_SD) {
    char buf[256];
    if (resize)
      snprintf(buf, sizeof buf, "%lu %.7g %.7g %.7g %.7g %.7g %.7g %.7g\n", t, packing, se[0],
               se[1], se[2], 0.5 * (se[1] + se[2]), se[3], se[4]);
    else
      snprintf(buf, sizeof buf, "%lu %.7g %.7g %.7g %.7g %.7g %.7g\n", t, se[0], se[1], se[2],
               0.5 * (se[1] + se[2]), se[3], se[4]);
    o << buf;
  } else {
    o << t << " ";
    if (resize) o << packing << " ";
    o << se[0] << " " << se[1] << " " << se[2] << " " << se[3] << "\n";
  }
}

// Open the stress/energy file: new at t_start == 0, else keep the lines up to the
// one of time t_start and continue after it (the reference's continue,
// strain_dynamics.cpp:248-279).
int open_se(sc::Handle& h, const std::string& path, unsigned long t_start, std::ofstream& out) {
  if (t_start == 0) {
    out.open(path, std::ios::out | std::ios::trunc);
    if (!out) return io_fail(&h, SC_E_IO, "cannot open " + path + " for writing");
    return SC_OK;
  }
  std::ifstream in(path);
  if (!in) return io_fail(&h, SC_E_IO, "cannot open " + path + " to continue");
  std::string line, kept;
  bool found = false;
  while (std::getline(in, line)) {
    kept += line + "\n";
    unsigned long t = std::strtoul(line.c_str(), nullptr, 10);
    if (!line.empty() && t == t_start) {
      found = true;
      break;
    }
  }
  in.close();
  if (!found) return io_fail(&h, SC_E_IO, "start time not found in " + path);
  out.open(path, std::ios::out | std::ios::trunc);
  if (!out) return io_fail(&h, SC_E_IO, "cannot rewrite " + path);
  out << kept;
  return SC_OK;
}

int check_single(sc_handle* H, const char* what) {
  if (!H) return SC_E_ARG;
  if (H->h.nsys != 1) return io_fail(&H->h, SC_E_ARG, std::string(what) + ": one system per handle");
  return SC_OK;
}

}  // namespace

extern "C" {

// Binary position file, save_positions_bin (src/cuda/strain_dynamics.cu:845-875).
static int read_bin(const char* path, int* n, double* hdr, double* x, double* y, double* phi,
                    double* R, double* A) {
  FILE* f = fopen(path, "rb");
  if (!f) return io_fail(nullptr, SC_E_IO, std::string("cannot open ") + path);
  int N = 0;
  double h[7];
  bool ok = fread(&N, sizeof N, 1, f) == 1 && fread(h, sizeof(double), 7, f) == 7 && N >= 0;
  if (!ok) {
    fclose(f);
    return io_fail(nullptr, SC_E_IO, std::string("short header in ") + path);
  }
  if (hdr) memcpy(hdr, h, sizeof h);
  if (!x) {
    fclose(f);
    *n = N;
    return SC_OK;
  }
  if (*n < N) {
    fclose(f);
    return io_fail(nullptr, SC_E_ARG, "arrays too short for the file");
  }
  for (int k = 0; k < N && ok; k++) {
    double v[5];
    ok = fread(v, sizeof(double), 5, f) == 5;
    if (ok) {
      x[k] = v[0];
      y[k] = v[1];
      phi[k] = v[2];
      R[k] = v[3];
      A[k] = v[4];
    }
  }
  fclose(f);
  if (!ok) return io_fail(nullptr, SC_E_IO, "fewer particles than the header's N");
  *n = N;
  return SC_OK;
}

// Whole content of a gzip-compressed file.  The reference's GzFileInput pipes the
// file through zcat (src/cpp/gz_file_input.cpp:76-78); here zlib is loaded at run
// time (libz.so.1, present wherever Python is), so neither a shell nor zlib's
// headers are needed to build.
static int read_gz(const char* path, std::string& out) {
  typedef void* (*open_fn)(const char*, const char*);
  typedef int (*read_fn)(void*, void*, unsigned);
  typedef int (*close_fn)(void*);
  static void* lib = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
  if (!lib) return io_fail(nullptr, SC_E_IO, "reading .gz files needs libz.so.1");
  auto gz_open = reinterpret_cast<open_fn>(dlsym(lib, "gzopen"));
  auto gz_read = reinterpret_cast<read_fn>(dlsym(lib, "gzread"));
  auto gz_close = reinterpret_cast<close_fn>(dlsym(lib, "gzclose"));
  if (!gz_open || !gz_read || !gz_close) return io_fail(nullptr, SC_E_IO, "libz.so.1 lacks gzopen");
  void* f = gz_open(path, "rb");
  if (!f) return io_fail(nullptr, SC_E_IO, std::string("cannot open ") + path);
  std::vector<char> buf(1 << 20);
  int got;
  while ((got = gz_read(f, buf.data(), (unsigned)buf.size())) > 0) out.append(buf.data(), got);
  gz_close(f);
  if (got < 0) return io_fail(nullptr, SC_E_IO, std::string("corrupt gzip data in ") + path);
  return SC_OK;
}

static int read_text(std::istream& in, const char* path, int* n, double* hdr, double* x,
                     double* y, double* phi, double* R, double* A);

int sc_read_positions(const char* path, int* n, double* hdr, double* x, double* y, double* phi,
                      double* R, double* A) {
  sc::g_noh_error.clear();
  if (!path || !n) return SC_E_ARG;
  const size_t plen = strlen(path);
  if (plen >= 4 && strcmp(path + plen - 4, ".bin") == 0) return read_bin(path, n, hdr, x, y, phi, R, A);
  if (plen >= 3 && strcmp(path + plen - 3, ".gz") == 0) {
    std::string text;
    int rc = read_gz(path, text);
    if (rc) return rc;
    std::istringstream in(text);
    return read_text(in, path, n, hdr, x, y, phi, R, A);
  }
  std::ifstream in(path);
  if (!in) return io_fail(nullptr, SC_E_IO, std::string("cannot open ") + path);
  return read_text(in, path, n, hdr, x, y, phi, R, A);
}

// DatFileInput with a header row (src/cpp/file_input.h:24-76) on either header layout
static int read_text(std::istream& in, const char* path, int* n, double* hdr, double* x,
                     double* y, double* phi, double* R, double* A) {
  std::string line;
  if (!std::getline(in, line)) return io_fail(nullptr, SC_E_IO, std::string("empty file ") + path);
  std::vector<double> head;
  {
    std::istringstream hs(line);
    double v;
    while (hs >> v) head.push_back(v);
  }
  if (head.size() != 7 && head.size() != 8)
    return io_fail(nullptr, SC_E_IO, "header must have 7 or 8 fields");
  int N = (int)head[0];
  double out_hdr[7];
  if (head.size() == 8) {
    for (int k = 0; k < 7; k++) out_hdr[k] = head[k + 1];
  } else {
    out_hdr[0] = out_hdr[1] = head[1];
    for (int k = 2; k < 7; k++) out_hdr[k] = head[k];
  }
  if (hdr) memcpy(hdr, out_hdr, sizeof out_hdr);
  if (!x) {
    *n = N;
    return SC_OK;
  }
  if (*n < N) return io_fail(nullptr, SC_E_ARG, "arrays too short for the file");
  int row = 0;
  while (row < N && std::getline(in, line)) {
    std::istringstream rs(line);
    double v[5];
    int k = 0;
    while (k < 5 && rs >> v[k]) k++;
    if (k == 0) continue;
    if (k < 5) return io_fail(nullptr, SC_E_IO, "short row in position file");
    x[row] = v[0];
    y[row] = v[1];
    phi[row] = v[2];
    R[row] = v[3];
    A[row] = v[4];
    row++;
  }
  if (row != N) return io_fail(nullptr, SC_E_IO, "fewer rows than the header's N");
  *n = N;
  return SC_OK;
}

// One position file from host arrays; head = Lx Ly packing gamma gamma_total rate dt.
// On failure *err says why.
static int write_positions(const char* path, int format, int n, const double head[7],
                           const double* x, const double* y, const double* p, const double* R,
                           const double* A, std::string* err) {
  const double Lx = head[0], Ly = head[1], packing = head[2];
  if (format == SC_FMT_BIN) {
    FILE* f = fopen(path, "wb");
    if (!f) return *err = std::string("cannot open ") + path, SC_E_IO;
    bool ok = fwrite(&n, sizeof n, 1, f) == 1 && fwrite(head, sizeof(double), 7, f) == 7;
    for (int k = 0; k < n && ok; k++) {
      const double v[5] = {x[k], y[k], p[k], R[k], A[k]};
      ok = fwrite(v, sizeof(double), 5, f) == 5;
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? SC_OK : (*err = std::string("write failed: ") + path, SC_E_IO);
  }
  if (format != SC_FMT_SP && format != SC_FMT_SD)
    return *err = "save_positions: unknown format", SC_E_ARG;
  if (format == SC_FMT_SD) {
    FILE* f = fopen(path, "w");
    if (!f) return *err = std::string("cannot open ") + path, SC_E_IO;
    fprintf(f, "%d %.17g %.17g %f %.17g %.14g %g %g\n", n, Lx, Ly, packing, head[3], head[4],
            head[5], head[6]);
    for (int k = 0; k < n; k++)
      fprintf(f, "%.17g %.17g %.17g %.2g %.17g\n", x[k], y[k], p[k], R[k], A[k]);
    bool ok = fclose(f) == 0;
    return ok ? SC_OK : (*err = std::string("write failed: ") + path, SC_E_IO);
  }
  std::ofstream o(path);
  if (!o) return *err = std::string("cannot open ") + path, SC_E_IO;
  o.precision(14);
  // the src/cpp header has one box length; a rectangular box (after a rotation or
  // pure shear) takes the src/cuda header's two, which the reader tells by its length
  o << n << " " << Lx << " ";
  if (Ly != Lx) o << Ly << " ";
  o << packing << " " << head[3] << " " << head[4] << " " << head[5] << " " << head[6]
    << std::endl;
  for (int k = 0; k < n; k++)
    o << x[k] << " " << y[k] << " " << p[k] << " " << R[k] << " " << A[k] << std::endl;
  o.close();
  return o ? SC_OK : (*err = std::string("write failed: ") + path, SC_E_IO);
}

int sc_save_positions(sc_handle* H, int sys, const char* path, int format) {
  if (!H || !path) return SC_E_ARG;
  sc::Handle& h = H->h;
  if (sys < 0 || sys >= h.nsys) return io_fail(&h, SC_E_ARG, "sc_save_positions: bad system");
  std::vector<double> x, y, p;
  int rc = system_state(H, sys, x, y, p);
  if (rc) return rc;
  if (!h.ensure_host_shapes()) return h.last_status;
  const sc::HostSys& S = h.hs[sys];
  double packing = S.packing * (h.hs[sys].Lx > 0 ? 1.0 : 0.0);
  const double head[7] = {S.Lx, S.Ly, packing, S.gamma, S.gamma_total, S.strain_rate, S.step};
  std::string err;
  rc = write_positions(path, format, S.n, head, x.data(), y.data(), p.data(), h.h_R.data() + S.p0,
                       h.h_A.data() + S.p0, &err);
  return rc ? io_fail(&h, rc, err) : SC_OK;
}

int sc_write_positions(const char* path, int format, int n, const double* hdr, const double* x,
                       const double* y, const double* phi, const double* R, const double* A) {
  sc::g_noh_error.clear();
  if (!path || !hdr || n < 0 || (n > 0 && (!x || !y || !phi || !R || !A))) {
    sc::g_noh_error = "sc_write_positions: needs a path, a header and n >= 0 rows";
    return SC_E_ARG;
  }
  std::string err;
  int rc = write_positions(path, format, n, hdr, x, y, phi, R, A, &err);
  if (rc) sc::g_noh_error = err;
  return rc;
}

int sc_run_strain(sc_handle* H, const char* out_dir, double run_gamma, double pos_save,
                  double se_save, unsigned long t_start, int format, unsigned long* t_end) {
  int rc = check_single(H, "sc_run_strain");
  if (rc) return rc;
  sc::Handle& h = H->h;
  sc::HostSys& S = h.hs[0];
  if (!out_dir || !(S.strain_rate != 0) || !(S.step > 0) || !(run_gamma >= 0))
    return io_fail(&h, SC_E_ARG, "sc_run_strain: needs an output directory, rate != 0, dt > 0");
  if (format != SC_FMT_SP && format != SC_FMT_SD)
    return io_fail(&h, SC_E_ARG, "sc_run_strain: format must be SC_FMT_SP or SC_FMT_SD");
  const double rate = S.strain_rate, dt = S.step;
  // the drivers' clamps, src/cpp/main.cpp:87-90
  if (se_save < rate * dt) se_save = rate * dt;
  if (pos_save < rate) pos_save = rate;
  const long nT = (long)(run_gamma / rate + 0.5);
  const int nInt = (int)(1.0 / dt + 0.5);
  const long nPos = std::max(1L, (long)(pos_save / rate + 0.5));
  const int nSE = std::max(1, (int)(se_save / (rate * dt) + 0.5));
  const std::string dir(out_dir);
  const char* prefix = format == SC_FMT_SD ? "sd" : "sp";
  const std::string se_path = dir + (format == SC_FMT_SD ? "/sd_stress_energy.dat" : "/sp_strain_se.dat");
  std::ofstream se_out;
  if ((rc = open_se(h, se_path, t_start, se_out))) return rc;
  double se[5] = {0, 0, 0, 0, 0};
  if (t_start == 0) {
    if ((rc = sc_calc_se(H, se))) return rc;
    se_line(se_out, format, 0, se, false, 0);
    if ((rc = sc_save_positions(H, 0, pos_name(dir, prefix, 0).c_str(), format))) return rc;
  } else if ((rc = sc_calc_forces(H))) {
    return rc;
  }
  std::vector<double> rec((size_t)(nInt / nSE + 1) * 5);
  for (unsigned long t = t_start + 1; t <= t_start + (unsigned long)nT; t++) {
    rc = h.run_steps(sc::KIND_STRAIN, 0, nInt, nSE, rec.data());
    if (rc) return rc;
    for (int k = 0; k < nInt / nSE; k++) {
      memcpy(se, &rec[5 * (size_t)k], sizeof se);
      se_line(se_out, format, t, se, false, 0);
    }
    if ((t * (unsigned long)nInt) % (unsigned long)nSE == 0) se_line(se_out, format, t, se, false, 0);
    if (t % (unsigned long)nPos == 0) {
      se_out.flush();
      if ((rc = sc_save_positions(H, 0, pos_name(dir, prefix, t).c_str(), format))) return rc;
    }
  }
  se_out.close();
  unsigned long tend = t_start + (unsigned long)nT;
  if ((rc = sc_save_positions(H, 0, pos_name(dir, prefix, tend).c_str(), format))) return rc;
  if (t_end) *t_end = tend;
  return SC_OK;
}

int sc_run_resize(sc_handle* H, const char* out_dir, double final_packing, double pos_save,
                  double se_save, unsigned long t_start, int format, unsigned long* t_end) {
  int rc = check_single(H, "sc_run_resize");
  if (rc) return rc;
  sc::Handle& h = H->h;
  if (!out_dir || !(h.hs[0].resize_rate > 0 && h.hs[0].resize_rate < 1) || !(h.hs[0].step > 0) ||
      !(final_packing > 0))
    return io_fail(&h, SC_E_ARG, "sc_run_resize: needs an output directory, 0 < rate < 1, dt > 0");
  if (format != SC_FMT_SP && format != SC_FMT_SD)
    return io_fail(&h, SC_E_ARG, "sc_run_resize: format must be SC_FMT_SP or SC_FMT_SD");
  const double rate = h.hs[0].resize_rate, dt = h.hs[0].step;
  if (se_save < rate * dt) se_save = rate * dt;  // src/cpp/main_resize.cpp:283-286
  if (pos_save < rate) pos_save = rate;
  const int nInt = (int)(1.0 / dt + 0.5);
  const long nPos = std::max(1L, (long)(pos_save / rate + 0.5));
  const int nSE = std::max(1, (int)(se_save / (rate * dt) + 0.5));
  const std::string dir(out_dir);
  const char* prefix = format == SC_FMT_SD ? "sd" : "sp";
  const std::string se_path = dir + "/sp_resize_se.dat";
  // resize_box, resize_dynamics.cpp:246-330: packing follows the box area
  const double parea = h.hs[0].packing * (h.hs[0].Lx * h.hs[0].Ly);
  auto packing = [&]() { return parea / (h.hs[0].Lx * h.hs[0].Ly); };
  const bool shrink = final_packing > packing();
  std::ofstream se_out;
  if ((rc = open_se(h, se_path, t_start, se_out))) return rc;
  double se[5] = {0, 0, 0, 0, 0};
  if (t_start == 0) {
    if ((rc = sc_calc_se(H, se))) return rc;
    se_line(se_out, format, 0, se, true, packing());
    if ((rc = sc_save_positions(H, 0, pos_name(dir, prefix, 0).c_str(), format))) return rc;
  } else if ((rc = sc_calc_forces(H))) {
    return rc;
  }
  unsigned long t = t_start;
  while (shrink ? final_packing > packing() : final_packing < packing()) {
    t += 1;
    // in segments of nSE steps so the packing of each record is the host's exact one
    int done = 0;
    while (done < nInt) {
      int seg = std::min(nSE - (done % nSE), nInt - done);
      bool rec_here = (done + seg) % nSE == 0;
      double r5[5];
      rc = h.run_steps(sc::KIND_RESIZE, shrink ? 1 : 0, seg, rec_here ? seg : 0, rec_here ? r5 : nullptr);
      if (rc) return rc;
      done += seg;
      if (rec_here) {
        memcpy(se, r5, sizeof se);
        se_line(se_out, format, t, se, true, packing());
      }
    }
    h.hs[0].packing = packing();
    if ((t * (unsigned long)nInt) % (unsigned long)nSE == 0) se_line(se_out, format, t, se, true, packing());
    if (t % (unsigned long)nPos == 0) {
      se_out.flush();
      if ((rc = sc_save_positions(H, 0, pos_name(dir, prefix, t).c_str(), format))) return rc;
    }
  }
  se_out.close();
  if ((rc = sc_save_positions(H, 0, pos_name(dir, prefix, t).c_str(), format))) return rc;
  if (t_end) *t_end = t;
  return SC_OK;
}

// run_pure_strain_2p, src/cuda/2point_dynamics.cu:2286-2391: pure shear in whole
// time units (1/dt steps) until Lx/Ly reaches stop_aspect.  A negative rate is
// taken as its magnitude.  Stress/energy lines describe the state after N steps for
// every N that is a multiple of the stress interval, labelled with the time unit
// that N falls in; at each position save the line and the position file describe
// the state at the start of the unit.  The run ends with a line and a position file
// of the final state (the reference takes one more simple-shear step to write
// them, :2389).
int sc_run_pure_strain(sc_handle* H, const char* out_dir, double stop_aspect, double pos_save,
                       double se_save, unsigned long t_start, int format, unsigned long* t_end) {
  int rc = check_single(H, "sc_run_pure_strain");
  if (rc) return rc;
  sc::Handle& h = H->h;
  // h.hs is reassigned by every run_steps call: read it afresh each time
  auto box_aspect = [&]() { return h.hs[0].Lx / h.hs[0].Ly; };
  if (!out_dir || !(h.hs[0].strain_rate != 0) || !(h.hs[0].step > 0) || !(stop_aspect > 0))
    return io_fail(&h, SC_E_ARG,
                   "sc_run_pure_strain: needs an output directory, a non-zero rate, dt > 0");
  if (format != SC_FMT_SP && format != SC_FMT_SD)
    return io_fail(&h, SC_E_ARG, "sc_run_pure_strain: format must be SC_FMT_SP or SC_FMT_SD");
  if (h.hs[0].strain_rate < 0) {  // :2294-2297
    h.hs[0].strain_rate = -h.hs[0].strain_rate;
    h.pred_valid = false;
  }
  if (box_aspect() > stop_aspect)
    return io_fail(&h, SC_E_ARG,
                   "sc_run_pure_strain: the box aspect is already beyond the stop aspect");
  const double rate = h.hs[0].strain_rate, dt = h.hs[0].step;
  if (se_save < rate * dt) se_save = rate * dt;  // :2306-2309
  if (pos_save < rate) pos_save = rate;
  const unsigned long nInt = (unsigned long)(1.0 / dt + 0.5);
  const unsigned long nSE = std::max(1UL, (unsigned long)(se_save / (rate * dt) + 0.5));
  const unsigned long nPos = std::max(1UL, (unsigned long)(pos_save / rate + 0.5));
  const std::string dir(out_dir);
  const char* prefix = format == SC_FMT_SD ? "sd" : "sp";
  const std::string se_path = dir + (format == SC_FMT_SD ? "/sd_stress_energy.dat" : "/sp_strain_se.dat");
  std::ofstream se_out;
  if ((rc = open_se(h, se_path, t_start, se_out))) return rc;
  double se[5] = {0, 0, 0, 0, 0};
  bool have_top = false;  // se holds the record of the state at the unit's start
  unsigned long t = t_start;
  std::vector<double> rec;
  while (box_aspect() < stop_aspect) {
    const unsigned long N0 = t * nInt;
    const bool pos_here = t % nPos == 0;
    if (!(t == t_start && t_start > 0) && (pos_here || N0 % nSE == 0)) {
      // the continued line and position file of t_start are already written
      if (!have_top && (rc = sc_calc_se(H, se))) return rc;
      se_line(se_out, format, t, se, false, 0);
      if (pos_here) {
        se_out.flush();
        if ((rc = sc_save_positions(H, 0, pos_name(dir, prefix, t).c_str(), format))) return rc;
      }
    }
    have_top = false;
    unsigned long done = 0;
    while (done < nInt) {
      const unsigned long N = N0 + done;
      unsigned long seg, every;
      if (N % nSE == 0 && nSE <= nInt - done) {
        seg = ((nInt - done) / nSE) * nSE;  // whole record intervals in one call
        every = nSE;
      } else {
        seg = std::min(nSE - N % nSE, nInt - done);  // up to the next record (or unit end)
        every = (N + seg) % nSE == 0 ? seg : 0;
      }
      const unsigned long nrec = every ? seg / every : 0;
      rec.assign(nrec * 5 + 5, 0.0);
      rc = h.run_steps(sc::KIND_PURE, 0, (int)seg, (int)every, nrec ? rec.data() : nullptr);
      if (rc) return rc;
      for (unsigned long k = 0; k < nrec; k++) {
        const unsigned long Nk = N + (k + 1) * every;
        if (Nk == N0 + nInt) {
          memcpy(se, &rec[5 * k], sizeof se);  // the next unit's opening record
          have_top = true;
        } else {
          se_line(se_out, format, t, &rec[5 * k], false, 0);
        }
      }
      done += seg;
    }
    t += 1;
  }
  if (!have_top && (rc = sc_calc_se(H, se))) return rc;
  se_line(se_out, format, t, se, false, 0);
  se_out.close();
  if ((rc = sc_save_positions(H, 0, pos_name(dir, prefix, t).c_str(), format))) return rc;
  if (t_end) *t_end = t;
  return SC_OK;
}

// find_jam_2p with its output (src/cuda/2point_dynamics.cu:4393-4456, 4582-4606), and
// y_compress_energy_2p (:4458-4530, 4608-4631) with y_only: the start's position
// file, then per resize a stress/energy line "t packing E Pxx Pyy Pxy Pyx" in
// sd_stress_energy.dat and a position file, and the final state as a binary file.
// One system per handle.  As there, e_jam and the lines' energy column are
// calc_fe_2p's energy per unit area, and each resize relaxes with the conjugate
// gradient (cjpr_relax_2p, up to max_iter iterations) in the FP64 form; the mixed
// form relaxes with FIRE to ftol.
static int run_jam_files(sc_handle* H, const char* what, const char* out_dir, double e_jam,
                         double step, double min_step, double ftol, int max_iter, bool y_only,
                         int* steps_out, double* phi_jam) {
  int rc = check_single(H, what);
  if (rc) return rc;
  sc::Handle& h = H->h;
  if (!out_dir) return io_fail(&h, SC_E_ARG, std::string(what) + ": needs an output directory");
  const std::string dir(out_dir);
  std::ofstream se_out(dir + "/sd_stress_energy.dat");
  if (!se_out) return io_fail(&h, SC_E_IO, "cannot open " + dir + "/sd_stress_energy.dat");
  if ((rc = sc_save_positions(H, 0, pos_name(dir, "sd", 0).c_str(), SC_FMT_SD))) return rc;
  auto each = [&](int t, const double* se) -> int {
    const sc::HostSys& q = h.hs[0];
    // the energy column in e_jam's units (per unit area), the stresses as calc_se
    const double e_area = se[0] * (double)q.n / (2.0 * q.Lx * q.Ly);
    char buf[256];
    snprintf(buf, sizeof buf, "%d %.10f %.9g %.9g %.9g %.9g %.9g\n", t, q.packing, e_area, se[1],
             se[2], se[3], se[4]);
    se_out << buf;
    se_out.flush();
    return sc_save_positions(H, 0, pos_name(dir, "sd", (unsigned long)t).c_str(), SC_FMT_SD);
  };
  int steps = 0;
  double phi = 0;
  rc = h.find_jam(e_jam, step, min_step, ftol, max_iter, 1000000, &phi, &steps, each,
                  h.prec == sc::PREC_FP64, true, y_only);
  if (rc) return rc;
  se_out.close();
  char bin[32];
  snprintf(bin, sizeof bin, "/sd%010d.bin", steps);
  if ((rc = sc_save_positions(H, 0, (dir + bin).c_str(), SC_FMT_BIN))) return rc;
  if (steps_out) *steps_out = steps;
  if (phi_jam) *phi_jam = phi;
  return SC_OK;
}

int sc_run_find_jam(sc_handle* H, const char* out_dir, double e_jam, double step,
                    double ftol, int max_iter, int* steps_out, double* phi_jam) {
  return run_jam_files(H, "sc_run_find_jam", out_dir, e_jam, step, 1e-15, ftol, max_iter, false,
                       steps_out, phi_jam);
}

// y_compress_energy_2p stops below a step of 1e-14 (find_jam_2p: 1e-15)
int sc_run_y_compress(sc_handle* H, const char* out_dir, double e_target, double step,
                      double ftol, int max_iter, int* steps_out, double* packing) {
  return run_jam_files(H, "sc_run_y_compress", out_dir, e_target, step, 1e-14, ftol, max_iter,
                       true, steps_out, packing);
}

// compress_qs2p / expand_qs2p (src/cuda/2point_dynamics.cu:4296-4391): relaxation,
// then affine resizes by the length factor 1 - step (1/(1 - step) to expand, as
// resize_step_2p) each followed by a relaxation, until the packing fraction reaches
// final_packing; the start and every resize give a line "t packing E Pxx Pyy Pxy
// Pyx" in sd_stress_energy.dat (E per unit area, as the find-jam run) and sd%010d.dat.
// Relaxation: the conjugate gradient (cjpr_relax_2p, max_iter iterations) in the
// FP64 form, FIRE to ftol in the mixed form.
int sc_run_qs_compress(sc_handle* H, const char* out_dir, double final_packing, double step,
                       double ftol, int max_iter, int* steps_out) {
  int rc = check_single(H, "sc_run_qs_compress");
  if (rc) return rc;
  sc::Handle& h = H->h;
  if (!out_dir) return io_fail(&h, SC_E_ARG, "sc_run_qs_compress: needs an output directory");
  step = std::fabs(step);
  if (!(step > 0 && step < 1) || !(final_packing > 0))
    return io_fail(&h, SC_E_ARG, "sc_run_qs_compress: need 0 < |step| < 1 and final_packing > 0");
  const std::string dir(out_dir);
  std::ofstream se_out(dir + "/sd_stress_energy.dat");
  if (!se_out) return io_fail(&h, SC_E_IO, "cannot open " + dir + "/sd_stress_energy.dat");
  const bool fp64 = h.prec == sc::PREC_FP64;
  auto relax = [&]() {
    int r = fp64 ? h.cg_minimize(max_iter, nullptr, nullptr, nullptr)
                 : h.fire_minimize(ftol, max_iter, 1e-2, 0.2, nullptr, nullptr, nullptr);
    return r == SC_E_NOCONV ? SC_OK : r;
  };
  double se[5];
  auto record = [&](int t) -> int {
    int r = h.calc(true, se);
    if (r) return r;
    if ((r = sc_save_positions(H, 0, pos_name(dir, "sd", (unsigned long)t).c_str(), SC_FMT_SD)))
      return r;
    const sc::HostSys& q = h.hs[0];
    char buf[256];
    // the start's line prints the packing with %f, the resizes' with %.9f
    snprintf(buf, sizeof buf, t == 0 ? "%d %f %g %g %g %g %g\n" : "%d %.9f %g %g %g %g %g\n", t,
             q.packing, se[0] * (double)q.n / (2.0 * q.Lx * q.Ly), se[1], se[2], se[3], se[4]);
    se_out << buf;
    se_out.flush();
    return SC_OK;
  };
  if ((rc = relax()) || (rc = record(0))) return rc;
  const bool compress = final_packing >= h.hs[0].packing;
  const double f = compress ? 1.0 - step : 1.0 / (1.0 - step);
  int t = 0;
  while (compress ? h.hs[0].packing < final_packing : h.hs[0].packing > final_packing) {
    t += 1;
    if ((rc = h.affine_scale(std::vector<double>{f})) || (rc = relax()) || (rc = record(t)))
      return rc;
  }
  if (steps_out) *steps_out = t;
  return SC_OK;
}

int sc_run_minimize(sc_handle* H, const char* out_dir, int max_steps, double e_min,
                    int pos_save_n, int* steps_taken) {
  int rc = check_single(H, "sc_run_minimize");
  if (rc) return rc;
  sc::Handle& h = H->h;
  if (!out_dir || max_steps < 0) return io_fail(&h, SC_E_ARG, "sc_run_minimize: bad arguments");
  if (h.prec != sc::PREC_FP64)
    return io_fail(&h, SC_E_STATE, "sc_run_minimize is the reference's FP64 protocol");
  const std::string dir(out_dir);
  const int nPos = std::max(1, pos_save_n);
  std::ofstream se_out(dir + "/sr_strain_se.dat");
  if (!se_out) return io_fail(&h, SC_E_IO, "cannot open " + dir + "/sr_strain_se.dat");
  double se[5];
  int s;
  bool zero = false;
  for (s = 0; s < max_steps; s++) {
    if ((rc = sc_calc_se(H, se))) return rc;
    se_out << s << " " << se[0] << " " << se[1] << " " << se[2] << " " << se[3] << std::endl;
    if (se[0] <= e_min) {
      if ((rc = sc_save_positions(H, 0, pos_name(dir, "sr", s).c_str(), SC_FMT_SP))) return rc;
      zero = true;
      break;
    } else if (s % nPos == 0) {
      if ((rc = sc_save_positions(H, 0, pos_name(dir, "sr", s).c_str(), SC_FMT_SP))) return rc;
    }
    if ((rc = h.gd_step(se, e_min))) return rc;
  }
  if (!zero) {
    if ((rc = sc_calc_se(H, se))) return rc;
    se_out << max_steps << " " << se[0] << " " << se[1] << " " << se[2] << " " << se[3] << std::endl;
    if ((rc = sc_save_positions(H, 0, pos_name(dir, "sr", max_steps).c_str(), SC_FMT_SP)))
      return rc;
  }
  if (steps_taken) *steps_taken = s;
  return h.check_status("sc_run_minimize") ? SC_OK : h.last_status;
}

}  // extern "C"
