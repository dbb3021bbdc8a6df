// sc_api.cpp -- extern "C" entry points of libspherocyl (include/spherocyl.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/spherocyl.h"
#include "sc_host.hpp"
#include "sc_internal.hpp"

namespace sc {
thread_local std::string g_noh_error;
}

namespace {

const double kRefPi = 3.14159265358979;  // src/cpp/spherocyl_box.cpp:12
std::string& g_create_error = sc::g_noh_error;

}  // namespace

extern "C" {

const char* sc_version(void) { return "spherocyls_gb300 0.1 (sm_103a)"; }

const char* sc_status_string(int status) {
  switch (status) {
    case SC_OK: return "ok";
    case SC_E_ARG: return "invalid argument";
    case SC_E_IO: return "file i/o error";
    case SC_E_NAN: return "non-finite state";
    case SC_E_OVERFLOW: return "capacity exceeded";
    case SC_E_NOCONV: return "not converged";
    case SC_E_TIMEOUT: return "device wait timed out";
    case SC_E_CUDA: return "cuda error";
    case SC_E_STATE: return "invalid state";
    case SC_E_NOMEM: return "out of memory";
  }
  return "unknown status";
}

void sc_default_options(sc_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof *opt);
  opt->precision = SC_PREC_FP64;
  opt->stress_mode = SC_STRESS_COMPAT;
  opt->device = 0;
  opt->max_nbrs = 0;
  opt->use_graphs = 1;
  opt->block = 0;
  opt->profile = 0;
  opt->contact_model = SC_CONTACT_ONE;
  opt->stage_inputs = 0;
}

const char* sc_last_error(const sc_handle* h) {
  if (!h) return g_create_error.c_str();
  return h->h.err.c_str();
}

int sc_create(const sc_options* opt_in, int n_sys, const int* n_per_sys, const double* L,
              const double* pad, const double* x, const double* y, const double* phi,
              const double* R, const double* A, sc_handle** out) {
  return sc_create_rect(opt_in, n_sys, n_per_sys, L, L, pad, x, y, phi, R, A, out);
}

int sc_create_rect(const sc_options* opt_in, int n_sys, const int* n_per_sys, const double* L,
                   const double* Ly, const double* pad, const double* x, const double* y,
                   const double* phi, const double* R, const double* A, sc_handle** out) {
  g_create_error.clear();
  if (!out) return SC_E_ARG;
  *out = nullptr;
  if (n_sys <= 0 || !n_per_sys || !L || !Ly || !x || !y || !phi || !R || !A) {
    g_create_error = "sc_create: missing arrays or n_sys <= 0";
    return SC_E_ARG;
  }
  sc_options opt;
  if (opt_in)
    opt = *opt_in;
  else
    sc_default_options(&opt);
  if (opt.precision != SC_PREC_FP64 && opt.precision != SC_PREC_MIXED) {
    g_create_error = "sc_create: unknown precision";
    return SC_E_ARG;
  }
  if (opt.block < 0 || opt.block > 128 || opt.block % 32 != 0) {
    g_create_error = "sc_create: block must be 0 or a multiple of 32 up to 128";
    return SC_E_ARG;
  }
  if (opt.contact_model != SC_CONTACT_ONE && opt.contact_model != SC_CONTACT_TWO) {
    g_create_error = "sc_create: unknown contact model";
    return SC_E_ARG;
  }
  if (opt.pass_kind < SC_PASS_AUTO || opt.pass_kind > SC_PASS_TILE || opt.tile_target < 0 ||
      opt.tile_target > 65536 || opt.cg_max_probes < 0 || opt.persist_steps < 0 ||
      opt.persist_steps > 1) {
    g_create_error = "sc_create: pass_kind, tile_target, cg_max_probes or persist_steps out of range";
    return SC_E_ARG;
  }
  long long ntot_ll = 0;
  for (int s = 0; s < n_sys; s++) {
    if (n_per_sys[s] < 2 || !(L[s] > 0) || !std::isfinite(L[s]) || !(Ly[s] > 0) ||
        !std::isfinite(Ly[s]) || (pad && !(pad[s] >= 0))) {
      char buf[160];
      snprintf(buf, sizeof buf, "sc_create: system %d needs n >= 2, L > 0 and pad >= 0", s);
      g_create_error = buf;
      return SC_E_ARG;
    }
    ntot_ll += n_per_sys[s];
  }
  if (ntot_ll > (1LL << 30)) {
    g_create_error = "sc_create: too many particles";
    return SC_E_ARG;
  }
  const int ntot = (int)ntot_ll;
  // The input checks and per system the largest R and A (set_particle,
  // src/cpp/spherocyl_box.cpp:216-219) on worker threads over slices of the caller's
  // arrays, while this thread sums each system's filled area in particle order
  // (calculate_packing_fraction :357-366; a dependent chain of additions).
  std::vector<double> rmax(n_sys, 0.0), amax(n_sys, 0.0), filled(n_sys, 0.0);
  {
    std::vector<int> p0s(n_sys + 1, 0);
    for (int s = 0; s < n_sys; s++) p0s[s + 1] = p0s[s] + n_per_sys[s];
    const unsigned hw = std::thread::hardware_concurrency();
    const int nthreads = ntot < (1 << 16) ? 1 : (int)std::min(8u, std::max(1u, hw));
    struct Part {
      int fin = 1, shp = 1;  // all finite; every R > 0 and A >= 0
      std::vector<double> rm, am;
    };
    std::vector<Part> parts(nthreads);
    auto scan = [&](int w) {
      Part& P = parts[w];
      P.rm.assign(n_sys, 0.0);
      P.am.assign(n_sys, 0.0);
      const int a0 = (int)((long long)ntot * w / nthreads);
      const int a1 = (int)((long long)ntot * (w + 1) / nthreads);
      int s = (int)(std::upper_bound(p0s.begin(), p0s.end(), a0) - p0s.begin()) - 1;
      int fin = 1, shp = 1;
      for (int i = a0; i < a1; i++) {
        while (i >= p0s[s + 1]) s++;
        const double r = R[i], a = A[i];
        fin &= (int)std::isfinite(x[i]) & (int)std::isfinite(y[i]) &
               (int)std::isfinite(phi[i]) & (int)std::isfinite(r) & (int)std::isfinite(a);
        shp &= (int)(r > 0) & (int)(a >= 0);
        if (a > P.am[s]) P.am[s] = a;
        if (r > P.rm[s]) P.rm[s] = r;
      }
      P.fin = fin;
      P.shp = shp;
    };
    std::vector<std::thread> workers;
    std::vector<char> on_worker(nthreads, 0);
    for (int w = 1; w < nthreads; w++) {
      try {
        workers.emplace_back(scan, w);
        on_worker[w] = 1;
      } catch (...) {  // no thread to be had: this slice is scanned here
      }
    }
    for (int w = 0; w < nthreads; w++)
      if (!on_worker[w]) scan(w);
    for (int s = 0, i = 0; s < n_sys; s++) {
      double f = 0.0;
      for (int k = 0; k < n_per_sys[s]; k++, i++) f += (kRefPi * R[i] + 4.0 * A[i]) * R[i];
      filled[s] = f;
    }
    for (auto& t : workers) t.join();
    bool finite = true, shapes = true;
    for (const Part& P : parts) {
      finite = finite && P.fin;
      shapes = shapes && P.shp;
      for (int s = 0; s < n_sys; s++) {
        rmax[s] = std::max(rmax[s], P.rm[s]);
        amax[s] = std::max(amax[s], P.am[s]);
      }
    }
    if (!finite) {
      g_create_error = "sc_create: non-finite input";
      return SC_E_NAN;
    }
    if (!shapes) {
      g_create_error = "sc_create: every R must be > 0 and every A >= 0";
      return SC_E_ARG;
    }
  }

  sc_handle* H = new (std::nothrow) sc_handle;
  if (!H) return SC_E_NOMEM;
  sc::Handle& h = H->h;
  h.opt = opt;
  h.device = opt.device;
  h.prec = opt.precision;
  h.block = opt.block > 0 ? opt.block : 128;
  h.nsys = n_sys;
  h.ntot = ntot;
  auto bail = [&](int code) {
    g_create_error = h.err.empty() ? std::string("sc_create failed") : h.err;
    delete H;
    return code;
  };
  if (!h.cuda_ok(cudaSetDevice(h.device), "cudaSetDevice")) return bail(SC_E_CUDA);
  if (!h.cuda_ok(cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking), "stream"))
    return bail(SC_E_CUDA);
  h.own_stream = true;
  h.use_pool = sc::device_pool(h.device) != nullptr;
  if (!h.cuda_ok(cudaMallocHost((void**)&h.h_pinned, (16 + 12 * (size_t)n_sys) * sizeof(int)),
                 "pinned"))
    return bail(SC_E_NOMEM);

  // per-system scalars; the per-particle constants are computed on the device
  h.hs.resize(n_sys);
  int p0 = 0;
  for (int s = 0; s < n_sys; s++) {
    sc::HostSys& S = h.hs[s];
    S.n = n_per_sys[s];
    S.p0 = p0;
    S.Lx = L[s];
    S.Ly = Ly[s];
    S.pad = pad ? pad[s] : 0.0;
    S.Amax = amax[s];
    S.Rmax = rmax[s];
    const double filled_s = filled[s];
    S.packing = filled_s / (S.Lx * S.Ly);
    S.configure(true);
    p0 += S.n;
  }

  // device arrays
  const size_t N = ntot;
  sc::Dev& d = h.d;
  d.ntot = ntot;
  d.nsys = n_sys;
  d.stress_mode = opt.stress_mode == SC_STRESS_VIRIAL ? sc::STRESS_VIRIAL : sc::STRESS_COMPAT;
  d.contact_model = opt.contact_model == SC_CONTACT_TWO ? 1 : 0;
  d.maxn = opt.max_nbrs > 0 ? opt.max_nbrs : 64;
  // the tile pass keeps slots below 2^27 in its entries (kTileInt)
  d.pass_kind = (opt.precision == SC_PREC_MIXED && opt.pass_kind == SC_PASS_TILE &&
                 N < (size_t)sc::kTileInt) ? 1 : 0;
  std::vector<int> pchunk_sys, pchunk_p0, pchunk_np;
  for (int s = 0; s < n_sys; s++) {
    const sc::HostSys& S = h.hs[s];
    for (int k = 0; k < S.n; k += sc::kSeChunk) {
      pchunk_sys.push_back(s);
      pchunk_p0.push_back(S.p0 + k);
      pchunk_np.push_back(std::min(sc::kSeChunk, S.n - k));
    }
  }
  d.npchunks = (int)pchunk_sys.size();
  bool ok = true;
  sc::SysGeom* geom = nullptr;
  int *psys = nullptr, *pcs = nullptr, *pcp = nullptr, *pcn = nullptr;
  ok = ok && h.dalloc(&geom, n_sys, "geom") && h.dalloc(&psys, N, "psys");
  ok = ok && h.dalloc(&d.xy, N, "xy") && h.dalloc(&d.ph, N, "ph") && h.dalloc(&d.ra, N, "ra") &&
       h.dalloc(&d.irc, N, "irc") && h.dalloc(&d.id, N, "id") && h.dalloc(&d.cell, N, "cell");
  ok = ok && h.dalloc(&d.nxy, N, "nxy") && h.dalloc(&d.xy_t, N, "xy_t") &&
       h.dalloc(&d.ph_t, N, "ph_t") && h.dalloc(&d.nxy_t, N, "nxy_t");
  ok = ok && h.dalloc(&d.v0x, N, "v0x") && h.dalloc(&d.v0y, N, "v0y") &&
       h.dalloc(&d.v0p, N, "v0p") && h.dalloc(&d.fx, N, "fx") && h.dalloc(&d.fy, N, "fy") &&
       h.dalloc(&d.tau, N, "tau") && h.dalloc(&d.moved, N, "moved");
  if (h.prec == sc::PREC_MIXED)
    ok = ok && h.dalloc(&d.rec, N, "rec") && h.dalloc(&d.rec_t, N, "rec_t") &&
         h.dalloc(&d.mc, N, "mc") && h.dalloc(&d.mv, N, "mv") && h.dalloc(&d.mm, N, "mm") &&
         h.dalloc(&d.pa, N, "pa") && h.dalloc(&d.rcf, N, "rcf") && h.dalloc(&d.rf, N, "rf") &&
         h.dalloc(&d.cellp, N, "cellp") && h.dalloc(&d.gbuild, n_sys, "gbuild") &&
         h.dalloc(&d.ord, N, "ord") && h.dalloc(&d.nbr_p, N * d.maxn, "nbr_p") &&
         h.dalloc(&d.nbr_pn, N, "nbr_pn");
  if (opt.precision == SC_PREC_MIXED) {
    ok = ok && h.dalloc(&d.gbar, 2, "grid barrier") && h.dalloc(&h.d_persist, 1, "persist out");
    if (ok) ok = h.cuda_ok(cudaMemsetAsync(d.gbar, 0, 2 * sizeof(unsigned), h.stream), "barrier");
  }
  if (d.pass_kind == 1)
    ok = ok && h.dalloc(&d.t_own, N * sc::kTileEPP, "tile owners") &&
         h.dalloc(&d.t_pe, N * sc::kTileEPP, "tile partners") &&
         h.dalloc(&d.t_rd, N * sc::kTileEPP, "tile reads") && h.dalloc(&d.t_meta, N, "tile meta") &&
         h.dalloc(&d.t_pb, N * sc::kTileEPP, "tile pair results");
  ok = ok && h.dalloc(&d.nbr, N * d.maxn, "nbr");
  ok = ok && h.dalloc(&d.nbr_n, N, "nbr_n");
  ok = ok && h.dalloc(&d.cell_tmp, N, "cell_tmp") && h.dalloc(&d.rank, N, "rank") &&
       h.dalloc(&d.perm, N, "perm");
  ok = ok && h.dalloc(&d.s_xy, N, "s_xy") && h.dalloc(&d.s_ph, N, "s_ph") &&
       h.dalloc(&d.s_ra, N, "s_ra") && h.dalloc(&d.s_irc, N, "s_irc") &&
       h.dalloc(&d.s_id, N, "s_id") && h.dalloc(&d.s_cell, N, "s_cell");
  ok = ok && h.dalloc(&d.se_part, 5 * N, "se_part") &&
       h.dalloc(&d.se_chunk, 5 * (size_t)d.npchunks, "se_chunk") &&
       h.dalloc(&d.se_sys, 5 * (size_t)n_sys, "se_sys");
  ok = ok && h.dalloc(&pcs, d.npchunks, "pchunk") && h.dalloc(&pcp, d.npchunks, "pchunk") &&
       h.dalloc(&pcn, d.npchunks, "pchunk");
  ok = ok && h.dalloc(&d.flags, n_sys, "flags") && h.dalloc(&d.istar, n_sys, "istar") &&
       h.dalloc(&d.any, 1, "any") && h.dalloc(&d.work, n_sys, "work") &&
       h.dalloc(&d.woff, n_sys + 1, "woff") && h.dalloc(&d.wcoff, n_sys + 1, "wcoff") &&
       h.dalloc(&d.nwork, 3, "nwork") &&
       h.dalloc(&d.status, 2, "status");
  if (!ok) return bail(h.last_status ? h.last_status : SC_E_NOMEM);
  d.geom = geom;
  d.psys = psys;
  d.pchunk_sys = pcs;
  d.pchunk_p0 = pcp;
  d.pchunk_np = pcn;

  // initial slots: the input order.  The ingest kernel reads the caller's arrays in
  // place where the GPU addresses pageable host memory (Grace's coherent link), else
  // from device copies staged in the stress-partials buffer (5 N doubles, unused
  // until the first pass).
  cudaStream_t st = h.stream;
  std::vector<int> sys_p0(n_sys + 1);
  std::vector<double> sys_L(2 * (size_t)n_sys);
  for (int s = 0; s < n_sys; s++) {
    sys_p0[s] = h.hs[s].p0;
    sys_L[2 * s] = h.hs[s].Lx;
    sys_L[2 * s + 1] = h.hs[s].Ly;
  }
  sys_p0[n_sys] = ntot;
  int* d_sys_p0 = nullptr;
  double* d_sys_L = nullptr;
  ok = h.dalloc(&d_sys_p0, n_sys + 1, "systems") && h.dalloc(&d_sys_L, 2 * (size_t)n_sys, "systems");
  if (!ok) return bail(h.last_status ? h.last_status : SC_E_NOMEM);
  int pageable = 0;
  cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, h.device);
  const double* src[5] = {x, y, phi, R, A};
  if (!pageable || opt.stage_inputs) {
    for (int k = 0; k < 5 && ok; k++) {
      ok = h.cuda_ok(cudaMemcpyAsync(d.se_part + (size_t)k * N, src[k], N * sizeof(double),
                                     cudaMemcpyDefault, st), "upload");
      src[k] = d.se_part + (size_t)k * N;
    }
  }
  ok = ok &&
       h.cuda_ok(cudaMemcpyAsync(d_sys_p0, sys_p0.data(), (n_sys + 1) * sizeof(int),
                                 cudaMemcpyHostToDevice, st), "upload") &&
       h.cuda_ok(cudaMemcpyAsync(d_sys_L, sys_L.data(), 2 * (size_t)n_sys * sizeof(double),
                                 cudaMemcpyHostToDevice, st), "upload");
  if (ok) {
    sc::launch_ingest(d, src[0], src[1], src[2], src[3], src[4], d_sys_p0, d_sys_L, psys, st);
    ok = h.cuda_ok(cudaGetLastError(), "ingest launch");
  }
  ok = ok &&
       h.cuda_ok(cudaMemcpyAsync(pcs, pchunk_sys.data(), d.npchunks * sizeof(int),
                                 cudaMemcpyHostToDevice, st), "upload") &&
       h.cuda_ok(cudaMemcpyAsync(pcp, pchunk_p0.data(), d.npchunks * sizeof(int),
                                 cudaMemcpyHostToDevice, st), "upload") &&
       h.cuda_ok(cudaMemcpyAsync(pcn, pchunk_np.data(), d.npchunks * sizeof(int),
                                 cudaMemcpyHostToDevice, st), "upload") &&
       h.cuda_ok(cudaMemsetAsync(d.moved, 0, N * sizeof(double2), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.flags, 0, n_sys * sizeof(int), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.istar, 0x7f, n_sys * sizeof(int), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.any, 0, sizeof(int), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.nwork, 0, 3 * sizeof(int), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.status, 0, 2 * sizeof(int), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.nbr_n, 0, N * sizeof(int), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.fx, 0, N * sizeof(double), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.fy, 0, N * sizeof(double), st), "memset") &&
       h.cuda_ok(cudaMemsetAsync(d.tau, 0, N * sizeof(double), st), "memset") &&
       h.cuda_ok(cudaStreamSynchronize(st), "upload sync");
  if (!ok) return bail(h.last_status);
  h.dfree(d_sys_p0);
  h.dfree(d_sys_L);
  if (!h.layout_cells() || !h.rebuild_all() || !h.check_status("create"))
    return bail(h.last_status);
  *out = H;
  return SC_OK;
}

int sc_destroy(sc_handle* h) {
  delete h;
  return SC_OK;
}

int sc_trim_memory(int device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return SC_E_ARG;
  }
  cudaMemPool_t pool = sc::device_pool(device);
  if (pool && cudaMemPoolTrimTo(pool, 0) != cudaSuccess) return SC_E_CUDA;
  return SC_OK;
}

int sc_set_stream(sc_handle* H, void* stream) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  cudaSetDevice(h.device);
  cudaStreamSynchronize(h.stream);
  if (h.own_stream && h.stream) cudaStreamDestroy(h.stream);
  if (stream) {
    h.stream = (cudaStream_t)stream;
    h.own_stream = false;
  } else {
    cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking);
    h.own_stream = true;
  }
  return SC_OK;
}

int sc_synchronize(sc_handle* H) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  cudaSetDevice(h.device);
  return h.check_status("synchronize") ? SC_OK : h.last_status;
}

static int set_scalar(sc_handle* H, int sys, double v, double sc::HostSys::*field, bool rebuild,
                      const char* what) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  if (sys < -1 || sys >= h.nsys || !std::isfinite(v)) {
    h.fail(SC_E_ARG, "%s: bad system index or value", what);
    return SC_E_ARG;
  }
  for (int s = 0; s < h.nsys; s++)
    if (sys < 0 || s == sys) h.hs[s].*field = v;
  h.pred_valid = false;
  if (rebuild) {
    cudaSetDevice(h.device);
    if (!h.rebuild_all() || !h.check_status(what)) return h.last_status;
  }
  return SC_OK;
}

int sc_set_strain_rate(sc_handle* h, int sys, double v) {
  return set_scalar(h, sys, v, &sc::HostSys::strain_rate, false, "sc_set_strain_rate");
}
int sc_set_resize_rate(sc_handle* h, int sys, double v) {
  return set_scalar(h, sys, v, &sc::HostSys::resize_rate, false, "sc_set_resize_rate");
}
int sc_set_step(sc_handle* h, int sys, double v) {
  return set_scalar(h, sys, v, &sc::HostSys::step, false, "sc_set_step");
}
// The neighbour criterion depends on gamma, so a new gamma rebuilds the lists.
int sc_set_gamma(sc_handle* h, int sys, double v) {
  return set_scalar(h, sys, v, &sc::HostSys::gamma, true, "sc_set_gamma");
}
int sc_set_total_gamma(sc_handle* h, int sys, double v) {
  return set_scalar(h, sys, v, &sc::HostSys::gamma_total, false, "sc_set_total_gamma");
}

// Mixed form: time the shear step of a throwaway copy of the handle (same state,
// scalars and options) for each padding factor and block size, then give the live
// handle the fastest pair.  The padding only trades list length against rebuild
// frequency: every pair that can touch stays in the list, so the physics is the
// same.  The FP64 form keeps the caller's padding (it sets the reference's rebuild
// timing) and is left alone.
int sc_autotune(sc_handle* H, int steps, double* pad_factor, int* block) {
  if (!H || steps < 1) return SC_E_ARG;
  sc::Handle& h = H->h;
  cudaSetDevice(h.device);
  if (pad_factor) *pad_factor = 1.0;
  if (!h.ensure_host_shapes()) return h.last_status;
  if (block) *block = h.block;
  if (h.prec != sc::PREC_MIXED) return SC_OK;
  const int n = h.ntot, ns = h.nsys;
  std::vector<double> x(n), y(n), p(n), L(ns), Ly(ns), pad0(ns), pads(ns);
  std::vector<int> nps(ns);
  int rc = sc_get_state(H, x.data(), y.data(), p.data());
  if (rc) return rc;
  for (int s = 0; s < ns; s++) {
    nps[s] = h.hs[s].n;
    L[s] = h.hs[s].Lx;
    Ly[s] = h.hs[s].Ly;
    pad0[s] = h.hs[s].pad;
  }
  // candidates: padding factor x (per-particle pass at two block sizes, or the
  // tile pass at three tile sizes)
  struct Cand {
    double f;
    int kind, block, target, persist;
  };
  std::vector<Cand> cands;
  for (double f : {0.5, 1.0, 1.5, 2.0, 3.0}) {
    for (int b : {64, 128}) cands.push_back({f, SC_PASS_LIST, b, 0, 0});
    cands.push_back({f, SC_PASS_LIST, 128, 0, 1});
    if (h.ntot < (int)sc::kTileInt)
      for (int t : {128, 256, 384}) cands.push_back({f, SC_PASS_TILE, h.block, t, 0});
  }
  Cand best{1.0, h.d.pass_kind == 1 ? SC_PASS_TILE : SC_PASS_LIST, h.block, h.opt.tile_target,
            h.opt.persist_steps};
  double best_ms = 1e300;
  cudaEvent_t e0, e1;
  if (!h.cuda_ok(cudaEventCreate(&e0), "event") || !h.cuda_ok(cudaEventCreate(&e1), "event"))
    return h.last_status;
  for (const Cand& c : cands) {
    sc_options o = h.opt;
    o.block = c.block;
    o.pass_kind = c.kind;
    o.tile_target = c.target;
    o.persist_steps = c.persist;
    o.profile = 0;
    for (int s = 0; s < ns; s++) pads[s] = c.f * pad0[s];
    sc_handle* T = nullptr;
    if (sc_create_rect(&o, ns, nps.data(), L.data(), Ly.data(), pads.data(), x.data(), y.data(),
                       p.data(), h.h_R.data(), h.h_A.data(), &T) != SC_OK)
      continue;  // e.g. out of memory for the copy: skip the candidate
    bool ok = true;
    for (int s = 0; s < ns && ok; s++) {
      const sc::HostSys& S = h.hs[s];
      ok = sc_set_strain_rate(T, s, S.strain_rate) == SC_OK &&
           sc_set_step(T, s, S.step) == SC_OK && sc_set_gamma(T, s, S.gamma) == SC_OK &&
           sc_set_total_gamma(T, s, S.gamma_total) == SC_OK;
    }
    float ms = 0.f;
    ok = ok && sc_strain_steps(T, steps, 0, nullptr) == SC_OK &&
         cudaEventRecord(e0, T->h.stream) == cudaSuccess &&
         sc_strain_steps(T, steps, 0, nullptr) == SC_OK &&
         cudaEventRecord(e1, T->h.stream) == cudaSuccess &&
         cudaEventSynchronize(e1) == cudaSuccess &&
         cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
    sc_destroy(T);
    if (ok && ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGetLastError();
  if (best_ms == 1e300) {
    h.fail(SC_E_CUDA, "sc_autotune: no candidate ran");
    return SC_E_CUDA;
  }
  const int kind = best.kind == SC_PASS_TILE ? 1 : 0;
  const bool relayout = best.f != 1.0 || kind != h.d.pass_kind ||
                        (kind == 1 && best.target != h.opt.tile_target);
  if (relayout) {
    if (!h.materialize()) return h.last_status;
    if (kind == 1 && !h.d.t_own) {
      const size_t N = h.ntot;
      if (!h.dalloc(&h.d.t_own, N * sc::kTileEPP, "tile owners") ||
          !h.dalloc(&h.d.t_pe, N * sc::kTileEPP, "tile partners") ||
          !h.dalloc(&h.d.t_rd, N * sc::kTileEPP, "tile reads") ||
          !h.dalloc(&h.d.t_meta, N, "tile meta") ||
          !h.dalloc(&h.d.t_pb, N * sc::kTileEPP, "tile pair results"))
        return h.last_status;
    }
    h.d.pass_kind = kind;
    h.opt.pass_kind = best.kind;
    h.opt.tile_target = best.target;
    for (int s = 0; s < ns; s++) {
      h.hs[s].pad = best.f * pad0[s];
      h.hs[s].configure(false);
    }
    if (!h.layout_cells() || !h.rebuild_all() || !h.check_status("sc_autotune"))
      return h.last_status;
  }
  h.block = best.block;
  h.opt.block = best.block;
  h.opt.persist_steps = best.persist;
  h.opt.pass_kind = best.kind;
  if (kind == 1) h.opt.tile_target = best.target;
  h.invalidate_graph();
  if (pad_factor) *pad_factor = best.f;
  if (block) *block = best.block;
  return SC_OK;
}

int sc_get_options(const sc_handle* H, sc_options* out) {
  if (!H || !out) return SC_E_ARG;
  *out = H->h.opt;
  return SC_OK;
}

int sc_find_neighbors(sc_handle* H) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  cudaSetDevice(h.device);
  if (!h.rebuild_all() || !h.check_status("sc_find_neighbors")) return h.last_status;
  return SC_OK;
}

int sc_calc_forces(sc_handle* H) {
  if (!H) return SC_E_ARG;
  return H->h.calc(false, nullptr);
}

int sc_calc_se(sc_handle* H, double* se_out) {
  if (!H) return SC_E_ARG;
  return H->h.calc(true, se_out);
}

int sc_strain_steps(sc_handle* H, int nsteps, int se_every, double* se_out) {
  if (!H) return SC_E_ARG;
  return H->h.run_steps(sc::KIND_STRAIN, 0, nsteps, se_every, se_out);
}

int sc_resize_steps(sc_handle* H, int nsteps, int shrink, int se_every, double* se_out) {
  if (!H) return SC_E_ARG;
  return H->h.run_steps(sc::KIND_RESIZE, shrink ? 1 : 0, nsteps, se_every, se_out);
}

int sc_pure_strain_steps(sc_handle* H, int nsteps, int se_every, double* se_out) {
  if (!H) return SC_E_ARG;
  return H->h.run_steps(sc::KIND_PURE, 0, nsteps, se_every, se_out);
}

int sc_gd_minimize(sc_handle* H, int max_steps, double e_min, int* steps_taken, double* e_final) {
  if (!H) return SC_E_ARG;
  if (max_steps < 0) {
    H->h.fail(SC_E_ARG, "max_steps must be >= 0");
    return SC_E_ARG;
  }
  if (H->h.prec != sc::PREC_FP64) {
    H->h.fail(SC_E_STATE, "sc_gd_minimize is the reference's FP64 protocol; use an FP64 handle");
    return SC_E_STATE;
  }
  return H->h.gd_minimize(max_steps, e_min, steps_taken, e_final);
}

// slot -> original index (systems concatenated)
int sc_get_state(sc_handle* H, double* x, double* y, double* phi) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  cudaSetDevice(h.device);
  if (!h.materialize()) return h.last_status;
  return h.read_unsorted(false, x, y, phi) ? SC_OK : h.last_status;
}

int sc_get_forces(sc_handle* H, double* fx, double* fy, double* tau) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  cudaSetDevice(h.device);
  // the mixed form's step passes do not keep the forces: evaluate them
  if (h.prec == sc::PREC_MIXED && !h.forces_valid) {
    int rc = h.calc(false, nullptr);
    if (rc) return rc;
  }
  return h.read_unsorted(true, fx, fy, tau) ? SC_OK : h.last_status;
}

int sc_get_box(sc_handle* H, int sys, double* out) {
  if (!H || !out) return SC_E_ARG;
  sc::Handle& h = H->h;
  if (sys < 0 || sys >= h.nsys) {
    h.fail(SC_E_ARG, "sc_get_box: bad system index");
    return SC_E_ARG;
  }
  const sc::HostSys& S = h.hs[sys];
  out[0] = S.Lx;
  out[1] = S.Ly;
  out[2] = S.gamma;
  out[3] = S.gamma_total;
  out[4] = S.pad;
  out[5] = S.Lx / S.cols;
  out[6] = S.Ly / S.rows;
  out[7] = S.packing;
  out[8] = S.rows;
  out[9] = S.cols;
  return SC_OK;
}

int sc_get_pairs(sc_handle* H, int sys, int* pairs, long cap, long* n_pairs) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  if (sys < 0 || sys >= h.nsys) {
    h.fail(SC_E_ARG, "sc_get_pairs: bad system index");
    return SC_E_ARG;
  }
  cudaSetDevice(h.device);
  sc::Dev& d = h.d;
  if (!h.check_status("sc_get_pairs")) return h.last_status;
  const sc::HostSys& S = h.hs[sys];
  std::vector<int> nn(S.n), ids(S.n), lst((size_t)S.n * d.maxn);
  if (!h.cuda_ok(cudaMemcpyAsync(nn.data(), d.nbr_n + S.p0, S.n * sizeof(int),
                                 cudaMemcpyDeviceToHost, h.stream), "read lists") ||
      !h.cuda_ok(cudaMemcpyAsync(ids.data(), d.id + S.p0, S.n * sizeof(int),
                                 cudaMemcpyDeviceToHost, h.stream), "read lists") ||
      !h.cuda_ok(cudaMemcpy2DAsync(lst.data(), S.n * sizeof(int), d.nbr + S.p0,
                                   (size_t)d.ntot * sizeof(int), S.n * sizeof(int), d.maxn,
                                   cudaMemcpyDeviceToHost, h.stream), "read lists") ||
      !h.cuda_ok(cudaStreamSynchronize(h.stream), "read lists"))
    return h.last_status;
  std::vector<std::pair<int, int>> pr;
  for (int k = 0; k < S.n; k++) {
    int c = std::min(nn[k], d.maxn);
    for (int m = 0; m < c; m++) {
      int j = (int)((unsigned)lst[(size_t)m * S.n + k] & sc::kSlotMask) - S.p0;
      if (j < 0 || j >= S.n) continue;
      int a = ids[k], b = ids[j];
      if (a < b) pr.emplace_back(a, b);
    }
  }
  std::sort(pr.begin(), pr.end());
  if (n_pairs) *n_pairs = (long)pr.size();
  if (pairs)
    for (long k = 0; k < (long)pr.size() && k < cap; k++) {
      pairs[2 * k] = pr[k].first;
      pairs[2 * k + 1] = pr[k].second;
    }
  return SC_OK;
}

int sc_fire_minimize(sc_handle* H, double ftol, int max_iter, double dt0, double dt_max,
                     int* iters, double* fmax, int* done) {
  if (!H) return SC_E_ARG;
  return H->h.fire_minimize(ftol, max_iter, dt0, dt_max, iters, fmax, done);
}

int sc_fire_iterations(const sc_handle* H, int* iters) {
  if (!H || !iters) return SC_E_ARG;
  const sc::Handle& h = H->h;
  for (int s = 0; s < h.nsys; s++) iters[s] = s < (int)h.fire_iters.size() ? h.fire_iters[s] : 0;
  return SC_OK;
}

int sc_strain_to_gamma(sc_handle* H, double gamma_max, long* steps) {
  if (!H) return SC_E_ARG;
  return H->h.strain_to_gamma(gamma_max, steps);
}

int sc_cg_minimize(sc_handle* H, int max_iter, int* iters, double* energy, int* reason) {
  if (!H) return SC_E_ARG;
  return H->h.cg_minimize(max_iter, iters, energy, reason);
}

int sc_flip_shear(sc_handle* H, int sys) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  if (sys < -1 || sys >= h.nsys) {
    h.fail(SC_E_ARG, "sc_flip_shear: bad system index");
    return SC_E_ARG;
  }
  std::vector<char> sel(h.nsys, 0);
  for (int s = 0; s < h.nsys; s++) sel[s] = sys < 0 || s == sys;
  return h.flip_shear(sel);
}

int sc_rotate_shear(sc_handle* H, int sys) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  if (sys < -1 || sys >= h.nsys) {
    h.fail(SC_E_ARG, "sc_rotate_shear: bad system index");
    return SC_E_ARG;
  }
  std::vector<char> sel(h.nsys, 0);
  for (int s = 0; s < h.nsys; s++) sel[s] = sys < 0 || s == sys;
  return h.rotate_shear(sel);
}

int sc_affine_scale(sc_handle* H, int sys, double factor) {
  if (!H) return SC_E_ARG;
  sc::Handle& h = H->h;
  if (sys < -1 || sys >= h.nsys || !(factor > 0) || !std::isfinite(factor)) {
    h.fail(SC_E_ARG, "sc_affine_scale: bad system index or factor");
    return SC_E_ARG;
  }
  std::vector<double> f(h.nsys, 1.0);
  for (int s = 0; s < h.nsys; s++)
    if (sys < 0 || s == sys) f[s] = factor;
  return h.affine_scale(f);
}

int sc_quasistatic_compress(sc_handle* H, double dphi, double ftol, double e_jam,
                            int max_increments, int max_iter, double* phi_jam, int* n_inc) {
  if (!H) return SC_E_ARG;
  return H->h.quasistatic(dphi, ftol, e_jam, max_increments, max_iter, phi_jam, n_inc);
}

int sc_find_jam(sc_handle* H, double e_jam, double step, double min_step, double ftol,
                int max_iter, int max_steps, double* phi_jam, int* steps) {
  if (!H) return SC_E_ARG;
  return H->h.find_jam(e_jam, step, min_step, ftol, max_iter, max_steps, phi_jam, steps);
}

int sc_get_counters(sc_handle* H, long long* out) {
  if (!H || !out) return SC_E_ARG;
  out[0] = H->h.steps;
  out[1] = H->h.dev_rebuilds;
  out[2] = H->h.dev_status;
  out[3] = H->h.kernels;
  return SC_OK;
}

int sc_get_pass_times(sc_handle* H, double* out) {
  if (!H || !out) return SC_E_ARG;
  sc::Handle& h = H->h;
  for (int k = 0; k < 3; k++) {
    out[k] = h.pass_n[k] ? h.pass_ms[k] / h.pass_n[k] : 0.0;
    out[3 + k] = (double)h.pass_n[k];
    h.pass_ms[k] = 0;
    h.pass_n[k] = 0;
  }
  return SC_OK;
}

}  // extern "C"
