// sc_host.cpp -- host runtime of libspherocyl: handle lifetime, device memory,
// per-step scalar tables, the step loops (eager or captured in CUDA graphs) and
// the C-ABI entry points declared in include/spherocyl.h.
//
// The host keeps an exact mirror of every per-system scalar the reference keeps
// (gamma, total gamma, box lengths, cell grid) and advances it with the
// reference's own floating-point operations (strain_step, resize_step and
// set_back_gamma: tmarschall/spherocyls src/cpp/strain_dynamics.cpp:231-234,
// src/cpp/resize_dynamics.cpp:230-238, src/cpp/spherocyl_box.cpp:542-543).  The
// device receives those values as tables, one row per step, so the only
// device-side decision is the displacement-triggered neighbour rebuild.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/spherocyl.h"
#include "sc_internal.hpp"
#include "sc_host.hpp"

namespace sc {

static const double kRefPi = 3.14159265358979;  // src/cpp/spherocyl_box.cpp:12

void Handle::fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  err = buf;
  last_status = code;
}

bool Handle::cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  fail(SC_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return false;
}

void Handle::dfree(void* p) {
  if (!p) return;
  auto it = std::find(allocs.begin(), allocs.end(), p);
  if (it != allocs.end()) allocs.erase(it);
  if (use_pool)
    cudaFreeAsync(p, stream);  // after the work already queued on the handle's stream
  else
    cudaFree(p);
}

cudaMemPool_t device_pool(int device) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lock(mu);
  auto it = pools.find(device);
  if (it != pools.end()) return it->second;
  cudaMemPool_t pool = nullptr;
  int supported = 0;
  if (cudaDeviceGetAttribute(&supported, cudaDevAttrMemoryPoolsSupported, device) ==
          cudaSuccess &&
      supported) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&pool, &props) == cudaSuccess) {
      // keep freed blocks: a handle created after another of the same size (a new
      // run, a copy for tuning) then costs no device allocation
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    } else {
      pool = nullptr;
    }
  }
  cudaGetLastError();  // a device without pools leaves no sticky error behind
  pools[device] = pool;
  return pool;
}

Handle::~Handle() {
  if (device >= 0) cudaSetDevice(device);
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  for (auto& c : sub_graphs) cudaGraphExecDestroy(c.exec);
  if (cg_exec) cudaGraphExecDestroy(cg_exec);
  if (stream2) cudaStreamDestroy(stream2);
  for (auto& e : ev_pool) cudaEventDestroy(e);
  if (use_pool) {
    for (void* p : allocs) cudaFreeAsync(p, stream);
    cudaStreamSynchronize(stream);
  } else {
    for (void* p : allocs) cudaFree(p);
  }
  if (h_pinned) cudaFreeHost(h_pinned);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

// ---- per-system geometry (set_particle and configure_cells on the host) ----

// configure_cells, src/cpp/spherocyl_box.cpp:223-241
void HostSys::configure(bool set_pad) {
  double wmin = wfac * (Rmax + Amax) + pad;
  double hmin = 2 * (Rmax + Amax) + pad;
  rows = std::max(static_cast<int>(Ly / hmin), 1);
  cols = std::max(static_cast<int>(Lx / wmin), 1);
  if (set_pad && pad == 0) pad = std::max(Lx / cols - wmin, Ly / rows - hmin);
}

// Whether the cell grid of the box (Lx_now, Ly_now) differs from the current one:
// reconfigure_cells' test (src/cpp/resize_dynamics.cpp:106-121, which takes the rows
// from Lx and the columns from Ly; the same for its square boxes) with rows from Ly
// and columns from Lx, the orientation configure() builds, so that the test is
// false right after a re-grid for rectangular boxes too (reconfigure_cells(0.0) of
// pure_strain_step_2p, src/cuda/spherocyl_box.cpp:46-67, uses that orientation).
bool HostSys::grid_changes_xy(double Lx_now, double Ly_now) const {
  double wmin = wfac * (Rmax + Amax) + pad;
  double hmin = 2 * (Rmax + Amax) + pad;
  int r = std::max(static_cast<int>(Ly_now / hmin), 1);
  int c = std::max(static_cast<int>(Lx_now / wmin), 1);
  return r != rows || c != cols;
}

// FP32 copies of a row, for the mixed form
static void fill_f32(StepScalars& t) {
  t.f_gamma_c = (float)t.gamma_c;
  t.f_gamma_p = (float)t.gamma_p;
  t.f_Wc = (float)t.W_c;
  t.f_Hc = (float)t.H_c;
  t.f_Wp = (float)t.W_p;
  t.f_Hp = (float)t.H_p;
  t.f_rate = (float)t.rate;
  t.f_step = (float)t.step;
  if (t.mode == 1 || t.mode == 2) {
    t.f_gx = t.f_gy = (float)(t.mode == 1 ? t.scale - 1.0 : 1.0 / t.scale - 1.0);
  } else if (t.mode == 3) {
    t.f_gx = (float)(0.5 * t.step * t.rate);
    t.f_gy = (float)(-0.5 * t.step * t.rate);
  } else {
    t.f_gx = t.f_gy = 0.0f;
  }
}

StepScalars Handle::row_current(int s) const {
  const HostSys& h = hs[s];
  StepScalars t;
  std::memset(&t, 0, sizeof t);
  t.gamma_c = h.gamma + h.step * h.strain_rate;
  t.gamma_p = h.gamma;
  t.Lx_c = t.Lx_p = h.Lx;
  t.Ly_c = t.Ly_p = h.Ly;
  t.W_c = t.W_p = h.Lx / h.cols;
  t.H_c = t.H_p = h.Ly / h.rows;
  t.rate = h.strain_rate;
  t.step = h.step;
  t.scale = 1.0;
  return t;
}

// ---- device layout ----

bool Handle::layout_cells() {
  // cells, scan chunks and particle chunks for all systems
  int c = 0, ch = 0;
  std::vector<int> chunk_sys, chunk_c0, chunk_nc, cell_sys;
  std::vector<int4> tiles;
  // tiles of about tile_target particles for the tile pass (one tile per system
  // otherwise): square blocks of cells at the system's mean occupancy
  const double target = opt.tile_target > 0 ? opt.tile_target : 256.0;
  for (int s = 0; s < nsys; s++) {
    HostSys& h = hs[s];
    h.c0 = c;
    int nc = h.rows * h.cols;
    h.ntx = h.nty = 1;
    if (d.pass_kind == 1) {
      const double occ = (double)h.n / nc;
      const int side = std::max(1, (int)std::lround(std::sqrt(target / occ)));
      h.ntx = (h.cols + side - 1) / side;
      h.nty = (h.rows + side - 1) / side;
    }
    for (int ky = 0; ky < h.nty; ky++) {
      const int y0 = tile_lo(ky, h.rows, h.nty), hy = tile_lo(ky + 1, h.rows, h.nty) - y0;
      for (int kx = 0; kx < h.ntx; kx++) {
        const int x0 = tile_lo(kx, h.cols, h.ntx), wx = tile_lo(kx + 1, h.cols, h.ntx) - x0;
        tiles.push_back(make_int4(s, c + y0 * h.cols + hy * x0, hy * wx, 0));
      }
    }
    h.chunk0 = ch;
    h.nchunks = (nc + kScanChunk - 1) / kScanChunk;
    for (int k = 0; k < h.nchunks; k++) {
      chunk_sys.push_back(s);
      chunk_c0.push_back(c + k * kScanChunk);
      chunk_nc.push_back(std::min(kScanChunk, nc - k * kScanChunk));
    }
    for (int k = 0; k < nc; k++) cell_sys.push_back(s);
    c += nc;
    ch += h.nchunks;
  }
  int ncells = c, nchunks = ch;
  if (ncells > cell_cap) {
    dfree(d.cell_start);
    dfree(d.cell_count);
    dfree((void*)d.cell_sys);
    int cap = ncells + ncells / 4 + 64;
    int *cs = nullptr, *cn = nullptr, *csys = nullptr;
    if (!dalloc(&cs, cap, "cell_start") || !dalloc(&cn, cap, "cell_count") ||
        !dalloc(&csys, cap, "cell_sys"))
      return false;
    d.cell_start = cs;
    d.cell_count = cn;
    d.cell_sys = csys;
    cell_cap = cap;
  }
  if (nchunks > chunk_cap) {
    dfree(d.chunk_sum);
    dfree(d.chunk_off);
    dfree((void*)d.chunk_sys);
    dfree((void*)d.chunk_c0);
    dfree((void*)d.chunk_nc);
    int cap = nchunks + nchunks / 4 + 16;
    int *a = nullptr, *b = nullptr, *e = nullptr, *f = nullptr, *g = nullptr;
    if (!dalloc(&a, cap, "chunk_sum") || !dalloc(&b, cap, "chunk_off") ||
        !dalloc(&e, cap, "chunk_sys") || !dalloc(&f, cap, "chunk_c0") ||
        !dalloc(&g, cap, "chunk_nc"))
      return false;
    d.chunk_sum = a;
    d.chunk_off = b;
    d.chunk_sys = e;
    d.chunk_c0 = f;
    d.chunk_nc = g;
    chunk_cap = cap;
  }
  const int ntiles = (int)tiles.size();
  if (ntiles > tile_cap) {
    dfree((void*)d.tiles);
    dfree(d.tinfo);
    int cap = ntiles + ntiles / 4 + 16;
    int4 *a = nullptr, *b = nullptr;
    if (!dalloc(&a, cap, "tiles") || !dalloc(&b, cap, "tile info")) return false;
    d.tiles = a;
    d.tinfo = b;
    tile_cap = cap;
  }
  d.ntiles = ntiles;
  d.ncells = ncells;
  d.nchunks = nchunks;
  invalidate_graph();  // captured kernels hold the old layout
  std::vector<SysGeom> g(nsys);
  int pch = 0;
  for (int s = 0; s < nsys; s++) {
    const HostSys& h = hs[s];
    SysGeom& o = g[s];
    std::memset(&o, 0, sizeof o);
    o.n = h.n;
    o.p0 = h.p0;
    o.c0 = h.c0;
    o.cols = h.cols;
    o.rows = h.rows;
    o.ntx = h.ntx;
    o.nty = h.nty;
    o.chunk0 = h.chunk0;
    o.nchunks = h.nchunks;
    o.pch0 = pch;
    pch += (h.n + kSeChunk - 1) / kSeChunk;
    o.pad = h.pad;
    o.inv_n = 1.0 / h.n;
    o.smax = (float)(2.0 * (h.Rmax + h.Amax));
    o.fpad = (float)h.pad;
  }
  bool ok = cuda_ok(cudaMemcpyAsync((void*)d.geom, g.data(), nsys * sizeof(SysGeom),
                                    cudaMemcpyHostToDevice, stream), "upload geometry") &&
            cuda_ok(cudaMemcpyAsync((void*)d.cell_sys, cell_sys.data(), ncells * sizeof(int),
                                    cudaMemcpyHostToDevice, stream), "upload cell map") &&
            cuda_ok(cudaMemcpyAsync((void*)d.chunk_sys, chunk_sys.data(), nchunks * sizeof(int),
                                    cudaMemcpyHostToDevice, stream), "upload chunks") &&
            cuda_ok(cudaMemcpyAsync((void*)d.chunk_c0, chunk_c0.data(), nchunks * sizeof(int),
                                    cudaMemcpyHostToDevice, stream), "upload chunks") &&
            cuda_ok(cudaMemcpyAsync((void*)d.chunk_nc, chunk_nc.data(), nchunks * sizeof(int),
                                    cudaMemcpyHostToDevice, stream), "upload chunks") &&
            cuda_ok(cudaMemcpyAsync((void*)d.tiles, tiles.data(), ntiles * sizeof(int4),
                                    cudaMemcpyHostToDevice, stream), "upload tiles") &&
            cuda_ok(cudaMemsetAsync(d.tinfo, 0, ntiles * sizeof(int4), stream), "tile info");
  if (!ok) return false;
  // host copies must outlive the async copies
  return cuda_ok(cudaStreamSynchronize(stream), "layout sync");
}

// The step table holds at least a full chunk from its first allocation, so that a
// run of short calls (a warm-up) followed by long ones does not re-allocate it.  Its
// address is captured by the whole-chunk, FIRE and CG graphs, which are dropped when
// it moves; the sub-chunk graphs read their rows from the step window instead and
// stay valid.
bool Handle::ensure_table(int rows) {
  if (rows * nsys <= tab_cap) return true;
  dfree(d_tab);
  int cap = std::max(std::max(rows, kChunk + 1) * nsys, 2 * tab_cap);
  StepScalars* t = nullptr;
  if (!dalloc(&t, cap, "step table")) return false;
  d_tab = t;
  tab_cap = cap;
  invalidate_table_graphs();
  return true;
}

void Handle::invalidate_table_graphs() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  graph_exec = nullptr;
  graph_key = GraphKey{};
  if (cg_exec) cudaGraphExecDestroy(cg_exec);
  cg_exec = nullptr;
  cg_key_iter = -1;
  if (fire_exec) cudaGraphExecDestroy(fire_exec);
  fire_exec = nullptr;
  fire_key_iters = 0;
}

bool Handle::upload_table(const std::vector<StepScalars>& rows) {
  int nrows = (int)(rows.size() / nsys);
  if (!ensure_table(nrows)) return false;
  // the host table is a member, so it outlives the asynchronous copy
  h_tab = rows;
  for (auto& t : h_tab) fill_f32(t);
  return cuda_ok(cudaMemcpyAsync(d_tab, h_tab.data(), h_tab.size() * sizeof(StepScalars),
                                 cudaMemcpyHostToDevice, stream),
                 "upload step table");
}

bool Handle::check_status(const char* where) {
  if (!cuda_ok(cudaMemcpyAsync(h_pinned, d.status, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                               stream), "read status") ||
      !cuda_ok(cudaStreamSynchronize(stream), where))
    return false;
  int st = h_pinned[0];
  dev_rebuilds = h_pinned[1];
  dev_status |= st;
  if (st & ST_NAN) {
    fail(SC_E_NAN, "%s: a position or angle became non-finite", where);
    return false;
  }
  if (st & ST_NBR_OVERFLOW) {
    fail(SC_E_OVERFLOW, "%s: a neighbour list exceeded max_nbrs=%d", where, d.maxn);
    return false;
  }
  if (st & ST_CELL_OVERFLOW) {
    fail(SC_E_OVERFLOW, "%s: cell sort lost particles", where);
    return false;
  }
  if (st & ST_BARRIER_TIMEOUT) {
    fail(SC_E_TIMEOUT, "%s: a grid barrier of the persistent step kernel timed out", where);
    return false;
  }
  return true;
}

// mixed form: bring the FP64 copy of the state up to date
bool Handle::materialize() {
  if (prec != PREC_MIXED || fp64_valid) return true;
  std::vector<StepScalars> rows(nsys);
  for (int s = 0; s < nsys; s++) rows[s] = row_current(s);
  if (!upload_table(rows)) return false;
  launch_mx_materialize(d, d_tab, 0, true, stream);
  kernels += 1;
  fp64_valid = true;
  return cuda_ok(cudaGetLastError(), "materialize");
}

// State (x, y, phi) or forces (fx, fy, tau) in the caller's particle order: one
// device scatter by particle index, then one copy per requested array.
bool Handle::read_unsorted(bool forces, double* a, double* b, double* c) {
  if (!d_out3 && !dalloc(&d_out3, 3 * (size_t)ntot, "output staging")) return false;
  if (forces)
    launch_unsort_forces(d, d_out3, stream);
  else
    launch_unsort_state(d, d_out3, stream);
  kernels += 1;
  double* dst[3] = {a, b, c};
  for (int k = 0; k < 3; k++)
    if (dst[k] && !cuda_ok(cudaMemcpyAsync(dst[k], d_out3 + (size_t)k * ntot,
                                           (size_t)ntot * sizeof(double),
                                           cudaMemcpyDeviceToHost, stream),
                           "read output"))
      return false;
  return cuda_ok(cudaStreamSynchronize(stream), "read output");
}

// R and A in input order, read back from the device the first time a caller needs
// them on the host (file output, copies for tuning); the handle does not keep host
// copies from its creation.  Slots stay inside their system's range, and id is the
// index within the system.
bool Handle::ensure_host_shapes() {
  if ((int)h_R.size() == ntot) return true;
  std::vector<double2> ra(ntot);
  std::vector<int> id(ntot);
  if (!cuda_ok(cudaMemcpyAsync(ra.data(), d.ra, (size_t)ntot * sizeof(double2),
                               cudaMemcpyDeviceToHost, stream), "read shapes") ||
      !cuda_ok(cudaMemcpyAsync(id.data(), d.id, (size_t)ntot * sizeof(int),
                               cudaMemcpyDeviceToHost, stream), "read shapes") ||
      !cuda_ok(cudaStreamSynchronize(stream), "read shapes"))
    return false;
  h_R.assign(ntot, 0.0);
  h_A.assign(ntot, 0.0);
  for (int s = 0; s < nsys; s++) {
    const HostSys& S = hs[s];
    for (int i = S.p0; i < S.p0 + S.n; i++) {
      const int k = S.p0 + id[i];
      h_R[k] = ra[i].x;
      h_A[k] = ra[i].y;
    }
  }
  return true;
}

// full rebuild of every system at the current state (constructor / setters)
bool Handle::rebuild_all() {
  if (!materialize()) return false;
  std::vector<StepScalars> rows(nsys);
  for (int s = 0; s < nsys; s++) rows[s] = row_current(s);
  if (!upload_table(rows)) return false;
  launch_force_rebuild_all(d, stream);
  launch_rebuild(d, prec == PREC_MIXED, d_tab, 0, stream);
  pred_valid = false;
  rebuilds++;
  return cuda_ok(cudaGetLastError(), "rebuild launch");
}

void Handle::launch_pass(int mode, bool se, int row, bool fast) {
  kernels += (prec == PREC_MIXED && se) ? 3 : 1;  // mixed: the FP64 stress kernels
  Dev dd = d;
  dd.cond = (mode == PASS_CORR_STRAIN || mode == PASS_CORR_RESIZE) ? step_cond : 0;
  dd.skip = pass_skip;
  if (prec == PREC_MIXED)
    launch_pass_mixed(dd, mode, se, d_tab, row, stream, block);
  else
    launch_pass_fp64(dd, mode, se, d_tab, row, stream, fast);
}

cudaEvent_t Handle::next_event() {
  if (ev_used == (int)ev_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    ev_pool.push_back(e);
  }
  return ev_pool[ev_used++];
}

void Handle::timed(int kind, bool on, const std::function<void()>& f) {
  if (!on) {
    f();
    return;
  }
  cudaEvent_t a = next_event(), b = next_event();
  cudaEventRecord(a, stream);
  f();
  cudaEventRecord(b, stream);
  ev_marks.push_back({kind, a, b});
}

void Handle::collect_times() {
  if (ev_marks.empty()) return;
  cudaStreamSynchronize(stream);
  for (auto& m : ev_marks) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m.a, m.b);
    pass_ms[m.kind] += ms;
    pass_n[m.kind] += 1;
  }
  ev_marks.clear();
  ev_used = 0;
}

// One Heun step (row k of the uploaded table), strain or resize form, in three
// parts: the corrector pass, the rebuild body (run only when a system needs it;
// every kernel in it also exits at once when none does), the predictor pass.
void Handle::enqueue_corr(bool resize, int k, bool prof) {
  timed(0, prof, [&] { launch_pass(resize ? PASS_CORR_RESIZE : PASS_CORR_STRAIN, false, k); });
}

int Handle::enqueue_rebuild_body(bool resize, int k, bool prof, cudaStream_t st) {
  int n = 0;
  cudaStream_t keep = stream;
  stream = st;
  // the systems to rebuild (flagged, or setting gamma back at this row) first, so
  // that the kernels before the cell sort touch their slots only
  launch_rb_worklist(d, d_tab, k, st);
  if (prec == PREC_MIXED) {
    // FP64 positions of the systems about to be sorted or set back
    launch_mx_materialize(d, d_tab, k, false, st);
    n++;
  }
  if (!resize) {
    launch_setback(d, d_tab, k, st);
    n++;
  }
  timed(2, prof, [&] { launch_rebuild(d, prec == PREC_MIXED, d_tab, k, st, true); });
  n += prec == PREC_MIXED ? 13 : 11;
  stream = keep;
  return n;
}

void Handle::enqueue_pred(bool resize, int k, bool se, bool prof) {
  timed(1, prof, [&] { launch_pass(resize ? PASS_PRED_RESIZE : PASS_PRED_STRAIN, se, k); });
}

void Handle::enqueue_step(bool resize, int k, bool se, bool prof) {
  enqueue_corr(resize, k, prof);
  kernels += enqueue_rebuild_body(resize, k, prof, stream);
  enqueue_pred(resize, k, se, prof);
}

void Handle::invalidate_graph() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  graph_exec = nullptr;
  graph_key = GraphKey{};
  for (auto& c : sub_graphs) cudaGraphExecDestroy(c.exec);
  sub_graphs.clear();
  if (cg_exec) cudaGraphExecDestroy(cg_exec);
  cg_exec = nullptr;
  cg_key_iter = -1;
  if (fire_exec) cudaGraphExecDestroy(fire_exec);
  fire_exec = nullptr;
  fire_key_iters = 0;
}

// A conditional handle on the graph being captured on `stream`, reset to 0 at
// every launch of the graph.
cudaError_t Handle::new_cond_handle(cudaGraphConditionalHandle* h) {
  return new_cond_handle(h, 0);
}

cudaError_t Handle::new_cond_handle(cudaGraphConditionalHandle* h, unsigned int dflt) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t gcap = nullptr;
  cudaError_t e = cudaStreamGetCaptureInfo(stream, &cs, nullptr, &gcap, nullptr, nullptr, nullptr);
  if (e == cudaSuccess)
    e = cudaGraphConditionalHandleCreate(h, gcap, dflt, cudaGraphCondAssignDefault);
  return e;
}

// Inside a capture on `stream`: an IF (or WHILE) node on `hcond` after the work
// captured so far, whose body `body` records on stream2.
cudaError_t Handle::add_cond_body(cudaGraphConditionalHandle hcond,
                                  const std::function<int(cudaStream_t)>& body,
                                  cudaGraphConditionalNodeType type) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t gcap = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(stream, &cs, nullptr, &gcap, &deps, nullptr, &nd);
  if (e != cudaSuccess) return e;
  // zeroed raw storage: the struct's union has no default constructor in C++
  alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)] = {};
  cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cp_buf);
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hcond;
  cp.conditional.type = type;
  cp.conditional.size = 1;
  cudaGraphNode_t cn;
  e = cudaGraphAddNode(&cn, gcap, deps, nullptr, nd, &cp);
  if (e == cudaSuccess)
    e = cudaStreamUpdateCaptureDependencies(stream, &cn, nullptr, 1,
                                            cudaStreamSetCaptureDependencies);
  if (e != cudaSuccess) return e;
  cudaGraph_t bg = cp.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(stream2, bg, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  body_kernels = body(stream2);
  return cudaStreamEndCapture(stream2, &bg);
}

// Inside a capture on `stream` (the FIRE iterations, whose update kernel does not
// switch the node itself): k_pre_rebuild for table row `row` (systems that set gamma
// back, or a pending rebuild), then the conditional node it switches on; `body`
// enqueues the node's contents on stream2 and returns its kernel count.
cudaError_t Handle::capture_rebuild_node(int row, const std::function<int(cudaStream_t)>& body) {
  cudaGraphConditionalHandle hcond;
  cudaError_t e = new_cond_handle(&hcond);
  if (e != cudaSuccess) return e;
  launch_pre_rebuild(d, d_tab, row, hcond, stream);
  return add_cond_body(hcond, body);
}

// Capture the per-step sequence with the rebuild body inside a conditional graph
// node (skipped when no system needs a rebuild).  Returns false, with the capture
// ended, when any capture step fails.
bool Handle::capture_conditional(bool resize, int nsteps, const std::vector<char>& se,
                                 cudaGraph_t* out) {
  if (!stream2 && !cuda_ok(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking), "stream"))
    return false;
  if (!cuda_ok(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture"))
    return false;
  cudaError_t e = cudaSuccess;
  int r = 0;
  long long fixed = 0;
  for (int k = 1; k <= nsteps && e == cudaSuccess; k++) {
    // the corrector pass itself switches the step's rebuild node on
    cudaGraphConditionalHandle hcond;
    e = new_cond_handle(&hcond);
    if (e != cudaSuccess) break;
    step_cond = hcond;
    enqueue_corr(resize, k, false);
    step_cond = 0;
    e = add_cond_body(hcond,
                      [&](cudaStream_t st) { return enqueue_rebuild_body(resize, k, false, st); });
    if (e != cudaSuccess) break;
    enqueue_pred(resize, k, se[k] != 0, false);
    fixed += 2;
    if (se[k]) {
      enqueue_se_record(r++);
      fixed += 3;
    }
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(stream, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return false;
  }
  graph_kernels = fixed;
  *out = g;
  return true;
}

// Capture `nsteps` steps (rows 1..nsteps of the current table pointer; se[k]: step k
// records stress/energy) and instantiate them.  With conditional nodes the rebuild
// bodies run only when needed, else every step carries the (early-exiting) chain.
bool Handle::instantiate_steps(bool resize, int nsteps, const std::vector<char>& se,
                               cudaGraphExec_t* exec, long long* nkernels) {
  cudaGraph_t g = nullptr;
  long long k0 = kernels;
  graph_conditional = use_conditional && capture_conditional(resize, nsteps, se, &g);
  kernels = k0;
  if (!graph_conditional) {
    use_conditional = false;  // plain capture: the rebuild kernels exit early
    if (!cuda_ok(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal),
                 "begin capture"))
      return false;
    int r = 0;
    for (int k = 1; k <= nsteps; k++) {
      enqueue_step(resize, k, se[k] != 0, false);
      if (se[k]) enqueue_se_record(r++);
    }
    graph_kernels = kernels - k0;
    kernels = k0;
    body_kernels = 0;
    if (!cuda_ok(cudaStreamEndCapture(stream, &g), "end capture")) return false;
  }
  *exec = nullptr;
  cudaError_t e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  // upload now, so that the first launch does not carry the upload
  if (e == cudaSuccess) e = cudaGraphUpload(*exec, stream);
  if (!cuda_ok(e, "graph instantiate")) {
    if (*exec) cudaGraphExecDestroy(*exec);
    *exec = nullptr;
    return false;
  }
  *nkernels = graph_kernels;
  return true;
}

// Capture `nsteps` steps (rows 1..nsteps) as one graph; reused while the table
// pointer, the shapes and the step kind stay the same (the table contents change
// from call to call, the graph reads them from device memory).
bool Handle::run_graph(bool resize, int nsteps, int se_every) {
  if (nsteps % kGraphSteps == 0) return run_subgraphs(resize, nsteps, se_every);
  GraphKey key{resize, nsteps, se_every, prec};
  if (!graph_exec || !(key == graph_key)) {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    graph_key = GraphKey{};
    std::vector<char> se(nsteps + 1, 0);
    for (int k = 1; k <= nsteps; k++) se[k] = se_every > 0 && k % se_every == 0;
    long long nk = 0;
    if (!instantiate_steps(resize, nsteps, se, &graph_exec, &nk)) return false;
    graph_key = key;
    chunk_kernels = nk;
  }
  kernels += chunk_kernels;
  return cuda_ok(cudaGraphLaunch(graph_exec, stream), "graph launch");
}

// The chunk (rows 1..nsteps of the table, records of steps that are multiples of
// se_every) as nsteps / kGraphSteps launches of sub-chunk graphs.
// The sub-chunk graph of kGraphSteps steps of this kind with the records of `mask`,
// captured on first use against the step and record windows.
Handle::SubGraph* Handle::subgraph(bool resize, unsigned mask) {
  const int G = kGraphSteps;
  if (!d_win && (!dalloc(&d_win, (size_t)(G + 1) * nsys, "step window") ||
                 !dalloc(&d_win_se, (size_t)G * nsys * 5, "record window")))
    return nullptr;
  for (auto& c : sub_graphs)
    if (c.resize == resize && c.se_mask == mask && c.prec == prec) return &c;
  // capture against the windows: swap them in for the table and record buffer
  std::vector<char> se(G + 1, 0);
  for (int k = 1; k <= G; k++) se[k] = (mask >> (k - 1)) & 1u;
  StepScalars* tab_keep = d_tab;
  double* rec_keep = d_se_hist;
  d_tab = d_win;
  d_se_hist = d_win_se;
  SubGraph c{resize, mask, prec, nullptr, 0};
  bool ok = instantiate_steps(resize, G, se, &c.exec, &c.kernels);
  d_tab = tab_keep;
  d_se_hist = rec_keep;
  if (!ok) return nullptr;
  sub_graphs.push_back(c);
  return &sub_graphs.back();
}

bool Handle::run_subgraphs(bool resize, int nsteps, int se_every) {
  const int G = kGraphSteps;
  int rec = 0;
  for (int j = 0; j < nsteps / G; j++) {
    unsigned mask = 0;
    for (int k = 1; k <= G; k++)
      if (se_every > 0 && (j * G + k) % se_every == 0) mask |= 1u << (k - 1);
    SubGraph* sg = subgraph(resize, mask);
    if (!sg) return false;
    const int nrec = __builtin_popcount(mask);
    if (!cuda_ok(cudaMemcpyAsync(d_win, d_tab + (size_t)j * G * nsys,
                                 (size_t)(G + 1) * nsys * sizeof(StepScalars),
                                 cudaMemcpyDeviceToDevice, stream),
                 "step window") ||
        !cuda_ok(cudaGraphLaunch(sg->exec, stream), "graph launch"))
      return false;
    kernels += sg->kernels;
    if (nrec > 0) {
      if (!cuda_ok(cudaMemcpyAsync(d_se_hist + (size_t)rec * nsys * 5, d_win_se,
                                   (size_t)nrec * nsys * 5 * sizeof(double),
                                   cudaMemcpyDeviceToDevice, stream),
                   "record window"))
        return false;
      rec += nrec;
    }
  }
  return true;
}

bool Handle::ensure_se_hist(int nrec) {
  if (nrec * nsys * 5 <= se_hist_cap) return true;
  dfree(d_se_hist);
  int cap = std::max(nrec * nsys * 5, 2 * se_hist_cap);
  double* p = nullptr;
  if (!dalloc(&p, cap, "se history")) return false;
  d_se_hist = p;
  se_hist_cap = cap;
  invalidate_table_graphs();  // the sub-chunk graphs record into their own window
  return true;
}

void Handle::enqueue_se_record(int rec) {
  kernels += 3;
  launch_se_reduce(d, stream);
  launch_se_store(d, d_se_hist + (size_t)rec * nsys * 5, stream);
}

// ---- protocols ----

// Advance one system's host mirror by one step and fill its table row
// (strain_step, strain_dynamics.cpp:231-234 with set_back_gamma,
// spherocyl_box.cpp:542-543; resize_step, resize_dynamics.cpp:230-238;
// pure_strain_step_2p, src/cuda/2point_dynamics.cu:2233-2278).
static void advance(HostSys& h, int kind, int shrink, StepScalars& t) {
  std::memset(&t, 0, sizeof t);
  t.rate = h.strain_rate;
  t.step = h.step;
  t.gamma_c = h.gamma + h.step * h.strain_rate;
  t.Lx_c = h.Lx;
  t.Ly_c = h.Ly;
  t.W_c = h.Lx / h.cols;
  t.H_c = h.Ly / h.rows;
  t.scale = 1.0;
  if (kind == KIND_PURE) {
    // the corrector pass sees the predicted box; gamma stays, the box follows the
    // flow after the step
    t.mode = 3;
    t.gamma_c = h.gamma;
    t.Lx_c = h.Lx * (1 + 0.5 * h.step * h.strain_rate);
    t.Ly_c = h.Ly * (1 - 0.5 * h.step * h.strain_rate);
    t.W_c = t.Lx_c / h.cols;
    t.H_c = t.Ly_c / h.rows;
    h.Lx += 0.5 * h.step * h.strain_rate * h.Lx;
    h.Ly -= 0.5 * h.step * h.strain_rate * h.Ly;
    h.gamma_total += h.step * h.strain_rate;
  } else if (kind == KIND_RESIZE) {
    t.scale = std::pow(1.0 - h.resize_rate, h.step);
    t.mode = shrink ? 1 : 2;
    if (shrink) {
      h.Lx *= std::pow(1.0 - h.resize_rate, h.step);
      h.Ly *= std::pow(1.0 - h.resize_rate, h.step);
    } else {
      h.Lx /= std::pow(1.0 - h.resize_rate, h.step);
      h.Ly /= std::pow(1.0 - h.resize_rate, h.step);
    }
  } else {
    h.gamma += h.strain_rate * h.step;
    h.gamma_total += h.strain_rate * h.step;
    // set_back_gamma at gamma >= 1/2 (src/cpp); for a rectangular box the image
    // offset Lx/Ly takes the place of 1 (src/cuda/strain_dynamics.cu:712-713)
    const double r = h.Lx / h.Ly;
    if (h.setback && h.gamma >= 0.5 * r) {
      h.gamma -= r;
      h.gamma_total = static_cast<int>(h.gamma_total + 1) + h.gamma;
      t.setback = 1;
    }
  }
  t.gamma_p = h.gamma;
  t.Lx_p = h.Lx;
  t.Ly_p = h.Ly;
  t.W_p = h.Lx / h.cols;
  t.H_p = h.Ly / h.rows;
}

int Handle::run_steps(int kind, int shrink, int nsteps, int se_every, double* se_out) {
  if (nsteps < 0 || se_every < 0) {
    fail(SC_E_ARG, "nsteps and se_every must be >= 0");
    return SC_E_ARG;
  }
  if (nsteps == 0) return SC_OK;
  // resize and pure shear share the affine pass modes (the row's mode tells them
  // apart); only simple shear sets gamma back
  const bool resize = kind != KIND_STRAIN;
  if (kind == KIND_RESIZE) {
    for (int s = 0; s < nsys; s++)
      if (!(hs[s].resize_rate > 0 && hs[s].resize_rate < 1)) {
        fail(SC_E_ARG, "resize rate of system %d must be in (0, 1)", s);
        return SC_E_ARG;
      }
  }
  if (kind == KIND_PURE) {
    for (int s = 0; s < nsys; s++)
      if (!(hs[s].strain_rate != 0) || !(std::fabs(hs[s].strain_rate * hs[s].step) < 1)) {
        fail(SC_E_ARG, "pure shear of system %d needs 0 < |strain rate| < 1/dt", s);
        return SC_E_ARG;
      }
  }
  cudaSetDevice(device);
  // The first step call of a kind captures the plain sub-chunk graph of that kind,
  // whatever its length, so that later calls (a long run after a short warm-up) do
  // not pay the capture.
  if (opt.use_graphs && !opt.profile && use_conditional &&
      !(opt.persist_steps && prec == PREC_MIXED && d.pass_kind == 0 && kind == KIND_STRAIN) &&
      !subgraph(kind != KIND_STRAIN, 0u))
    cudaGetLastError();  // capture failed: the chunks fall back to eager launches
  int nrec_total = (se_every > 0) ? nsteps / se_every : 0;
  std::vector<double> se_host((size_t)nrec_total * nsys * 5);
  int done = 0, rec_done = 0;
  bool regridded = false;  // the last pass of the loop re-gridded without stepping
  while (done < nsteps) {
    // chunk length: at most kChunk steps, a multiple of the recording period when
    // possible, and ending before any system's cell grid would change
    // (reconfigure_cells, resize_dynamics.cpp:106-121; for pure shear
    // src/cuda/spherocyl_box.cpp:46-67)
    int want = std::min(nsteps - done, kChunk);
    if (se_every > 0 && want >= se_every) want = (want / se_every) * se_every;
    int nk = want;
    bool regrid = false;
    if (resize) {
      std::vector<HostSys> sim = hs;
      StepScalars tmp;
      for (int k = 0; k < want; k++) {
        bool change = false;
        for (int s = 0; s < nsys; s++)
          if (sim[s].grid_changes_xy(sim[s].Lx, sim[s].Ly)) change = true;
        if (change) {
          nk = k;
          regrid = true;
          break;
        }
        for (int s = 0; s < nsys; s++) advance(sim[s], kind, shrink, tmp);
      }
    }
    if (nk == 0) {
      // the grid changes before the next step: re-grid, rebuild, continue.  The
      // mixed form's positions are relative to the old grid's cell centres, so the
      // FP64 state is brought up to date before the grid changes.
      if (regridded) {
        // the new grid already matched the box: a second change means the test and
        // the grid disagree, which would repeat for ever
        fail(SC_E_STATE, "cell grid does not settle after a re-grid");
        return SC_E_STATE;
      }
      if (!materialize()) return last_status;
      for (int s = 0; s < nsys; s++) hs[s].configure(false);
      if (!layout_cells() || !rebuild_all()) return last_status;
      regridded = true;
      continue;
    }
    regridded = false;
    std::vector<HostSys> sim = hs;
    std::vector<StepScalars> rows((size_t)(nk + 1) * nsys);
    for (int s = 0; s < nsys; s++) {
      // row 0 primes the predictor of the first step, which scales like any step
      rows[s] = row_current(s);
      if (kind == KIND_RESIZE) {
        rows[s].scale = std::pow(1.0 - hs[s].resize_rate, hs[s].step);
        rows[s].mode = shrink ? 1 : 2;
      } else if (kind == KIND_PURE) {
        rows[s].mode = 3;
      }
    }
    for (int k = 1; k <= nk; k++)
      for (int s = 0; s < nsys; s++) advance(sim[s], kind, shrink, rows[(size_t)k * nsys + s]);
    if (!upload_table(rows)) return last_status;
    // records of this chunk: steps done+k with (done+k) % se_every == 0
    int first_rec = rec_done;
    int nrec = 0;
    for (int k = 1; k <= nk; k++)
      if (se_every > 0 && (done + k) % se_every == 0) nrec++;
    if (nrec > 0 && !ensure_se_hist(nrec)) return last_status;
    const int pkind = kind == KIND_PURE ? 4 : (resize ? (shrink ? 2 : 3) : 1);
    if (!pred_valid || pred_kind != pkind) {
      launch_pass(resize ? PASS_PRED_RESIZE : PASS_PRED_STRAIN, false, 0);
      pred_valid = true;
      pred_kind = pkind;
    }
    bool aligned = se_every == 0 || done % se_every == 0;
    const bool use_persist = opt.persist_steps && prec == PREC_MIXED && d.pass_kind == 0 &&
                             kind == KIND_STRAIN && !opt.profile && d_persist;
    bool use_graph = !use_persist && opt.use_graphs && !opt.profile && nk >= 16 && aligned;
    if (use_persist) {
      if (!run_persist(nk, done, se_every)) return last_status;
    } else if (use_graph) {
      if (!run_graph(resize, nk, se_every)) return last_status;
    } else {
      int r = 0;
      for (int k = 1; k <= nk; k++) {
        bool se = se_every > 0 && (done + k) % se_every == 0;
        enqueue_step(resize, k, se, opt.profile != 0);
        if (se) enqueue_se_record(r++);
      }
    }
    if (!cuda_ok(cudaGetLastError(), "step launch")) return last_status;
    if (nrec > 0) {
      if (!cuda_ok(cudaMemcpyAsync(se_host.data() + (size_t)first_rec * nsys * 5, d_se_hist,
                                   (size_t)nrec * nsys * 5 * sizeof(double),
                                   cudaMemcpyDeviceToHost, stream),
                   "read se records"))
        return last_status;
    }
    collect_times();
    long long rb0 = dev_rebuilds;
    if (!check_status(kind == KIND_PURE ? "pure shear steps"
                                        : (resize ? "resize steps" : "strain steps")))
      return last_status;
    if (use_graph && graph_conditional) kernels += (dev_rebuilds - rb0) * body_kernels;
    fp64_valid = prec != PREC_MIXED;
    forces_valid = false;
    hs = sim;
    rec_done += nrec;
    done += nk;
    steps += nk;
    if (regrid) {
      // mixed form: positions relative to the old grid's cell centres first
      if (!materialize()) return last_status;
      for (int s = 0; s < nsys; s++) hs[s].configure(false);
      if (!layout_cells() || !rebuild_all()) return last_status;
    }
  }
  if (se_out && nrec_total > 0)
    std::memcpy(se_out, se_host.data(), se_host.size() * sizeof(double));
  return SC_OK;
}

// Steps 1..nk of the uploaded table with the persistent step kernel: runs of steps
// without a stress record go to one cooperative launch, which returns at the first
// step whose corrector asks for a rebuild; that step's rebuild and predictor are
// launched here, and the next run starts after it.  Recording steps take the
// regular launches.  One host synchronisation per launch (to read where it ended).
bool Handle::run_persist(int nk, int done, int se_every) {
  int r = 0;
  for (int k = 1; k <= nk;) {
    int kp = nk;  // last step of the run without a record
    if (se_every > 0) {
      const int next = ((done + k + se_every - 1) / se_every) * se_every - done;
      kp = std::min(nk, next - 1);
    }
    if (kp >= k) {
      if (!launch_persist_steps(d, d_tab, k, kp - k + 1, d_persist, stream)) {
        cudaGetLastError();
        fail(SC_E_CUDA, "persistent step kernel: cooperative launch failed");
        return false;
      }
      kernels += 1;
      if (!cuda_ok(cudaMemcpyAsync(h_pinned + 3, d_persist, sizeof(int), cudaMemcpyDeviceToHost,
                                   stream), "persist result") ||
          !cuda_ok(cudaStreamSynchronize(stream), "persist result"))
        return false;
      const int v = h_pinned[3];
      const int m = v >> 1;
      if (m < 0 || m > kp - k + 1 || (m == kp - k + 1 && (v & 1))) {
        fail(SC_E_STATE, "persistent step kernel returned %d", v);
        return false;
      }
      k += m;
      if (v & 1) {  // step k's corrector ran; its rebuild and predictor follow
        kernels += enqueue_rebuild_body(false, k, false, stream);
        enqueue_pred(false, k, false, false);
        k++;
      }
      continue;
    }
    enqueue_step(false, k, true, false);  // a recording step
    enqueue_se_record(r++);
    k++;
  }
  return true;
}

int Handle::calc(bool se, double* se_out) {
  cudaSetDevice(device);
  std::vector<StepScalars> rows(nsys);
  for (int s = 0; s < nsys; s++) rows[s] = row_current(s);
  if (!upload_table(rows)) return last_status;
  launch_pass(PASS_FORCE, se, 0);
  forces_valid = true;
  if (se) {
    launch_se_reduce(d, stream);
    if (!cuda_ok(cudaMemcpyAsync(h_pinned + 8, d.se_sys, 5 * nsys * sizeof(double),
                                 cudaMemcpyDeviceToHost, stream),
                 "read se"))
      return last_status;
  }
  if (!check_status("calc")) return last_status;
  if (se && se_out) {
    const double* src = reinterpret_cast<const double*>(h_pinned + 8);
    for (int s = 0; s < nsys; s++)
      for (int k = 0; k < 5; k++) se_out[5 * s + k] = src[(size_t)k * nsys + s];
  }
  return SC_OK;
}

// One fixed-size gradient step (gradient_relax_step, relaxation_dynamics.cpp:11-31)
// for every system whose energy is still above e_min; a rebuild follows any step
// that moved a particle beyond pad/2.
int Handle::gd_step(const double* se_now, double e_min) {
  std::vector<StepScalars> rows(nsys);
  for (int q = 0; q < nsys; q++) {
    rows[q] = row_current(q);
    if (se_now && se_now[5 * q] <= e_min) rows[q].step = 0.0;  // this system has finished
  }
  if (!upload_table(rows)) return last_status;
  launch_gd_update(d, prec == PREC_MIXED, d_tab, 0, stream);
  launch_rebuild(d, prec == PREC_MIXED, d_tab, 0, stream);
  kernels += 12;
  pred_valid = false;
  return cuda_ok(cudaGetLastError(), "gd step") ? SC_OK : last_status;
}

int Handle::gd_minimize(int max_steps, double e_min, int* steps_taken, double* e_final) {
  // gradient_descent_minimize, relaxation_dynamics.cpp:33-85: calc_se, test,
  // then one fixed-size gradient step.
  cudaSetDevice(device);
  std::vector<double> se(5 * (size_t)nsys);
  int s;
  for (s = 0; s < max_steps; s++) {
    int rc = calc(true, se.data());
    if (rc) return rc;
    bool all_done = true;
    for (int q = 0; q < nsys; q++)
      if (!(se[5 * q] <= e_min)) all_done = false;
    if (all_done) break;
    rc = gd_step(se.data(), e_min);
    if (rc) return rc;
  }
  if (steps_taken) *steps_taken = s;
  if (e_final) {
    double emax = 0;
    for (int q = 0; q < nsys; q++) emax = std::max(emax, se[5 * q]);
    *e_final = emax;
  }
  return check_status("gd minimize") ? SC_OK : last_status;
}

// ---- FIRE minimiser, affine rescale, quasistatic compression ----

bool Handle::ensure_fire() {
  if (fire.vx) return true;
  double *vx = nullptr, *vy = nullptr, *vp = nullptr, *part = nullptr;
  FireSys* sys = nullptr;
  int* done = nullptr;
  if (!dalloc(&vx, ntot, "fire vx") || !dalloc(&vy, ntot, "fire vy") ||
      !dalloc(&vp, ntot, "fire vp") || !dalloc(&sys, nsys, "fire sys") ||
      !dalloc(&part, 4 * (size_t)d.npchunks, "fire partials") ||
      !dalloc(&done, nsys, "fire done"))
    return false;
  fire.done = done;
  fire.vx = vx;
  fire.vy = vy;
  fire.vp = vp;
  fire.sys = sys;
  fire.part = part;
  d.fvx = vx;  // the rebuild permutes the minimiser's velocities from now on
  d.fvy = vy;
  d.fvp = vp;
  invalidate_graph();
  return true;
}

// One FIRE iteration, eagerly: force pass, reductions and update, rebuild chain.
void Handle::enqueue_fire_iteration(double ftol, double dt_max) {
  const bool mixed = prec == PREC_MIXED;
  // converged systems keep their forces and state: their force passes are skipped
  pass_skip = fire.done;
  launch_pass(PASS_FORCE, false, 0, true);
  pass_skip = nullptr;
  launch_fire_iteration_tail(d, fire, ftol, dt_max, mixed, stream);
  // the mixed form moves only its FP32 local state: the flagged systems'
  // FP64 copies are refreshed before the cell sort reads them
  launch_rb_worklist(d, d_tab, 0, stream);
  if (mixed) launch_mx_materialize(d, d_tab, 0, false, stream);
  launch_rebuild(d, mixed, d_tab, 0, stream, true);
  kernels += 4 + (mixed ? 14 : 12);
}

// `iters` FIRE iterations as one CUDA graph: each is force pass, reductions and
// update, then the rebuild chain inside a conditional node that runs only when a
// system was flagged.  Captured once per (iters, ftol, dt_max) and relaunched;
// returns false (nothing launched) when the capture is not possible.
bool Handle::run_fire_graph(int iters, double ftol, double dt_max) {
  if (!use_conditional) return false;
  if (!fire_exec || fire_key_iters != iters || fire_key_ftol != ftol || fire_key_dtmax != dt_max) {
    if (fire_exec) cudaGraphExecDestroy(fire_exec);
    fire_exec = nullptr;
    fire_key_iters = 0;
    if (!stream2 && !cuda_ok(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking), "stream"))
      return false;
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    const bool mixed = prec == PREC_MIXED;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < iters && e == cudaSuccess; k++) {
      pass_skip = fire.done;  // converged systems: no force pass
      launch_pass(PASS_FORCE, false, 0, true);
      pass_skip = nullptr;
      launch_fire_iteration_tail(d, fire, ftol, dt_max, mixed, stream);
      e = capture_rebuild_node(0, [&](cudaStream_t st) {
        launch_rb_worklist(d, d_tab, 0, st);
        if (mixed) launch_mx_materialize(d, d_tab, 0, false, st);
        launch_rebuild(d, mixed, d_tab, 0, st, true);
        return mixed ? 14 : 12;
      });
    }
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(stream, &g);
    cudaGraphExec_t ex = nullptr;
    if (e == cudaSuccess && e2 == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    fire_exec = ex;
    fire_key_iters = iters;
    fire_key_ftol = ftol;
    fire_key_dtmax = dt_max;
    fire_graph_kernels = 5LL * iters;
  }
  kernels += fire_graph_kernels;
  return cuda_ok(cudaGraphLaunch(fire_exec, stream), "fire graph launch");
}

// `iters` FIRE iterations with the persistent kernel of the mixed form.  A launch
// returns after the iteration that asks for a rebuild, which is launched here before
// the next one (as the graph's conditional node does), or once every system has
// converged.  One host synchronisation per launch, to read where it ended.
bool Handle::run_persist_fire(int iters, double ftol, double dt_max) {
  for (int k = 0; k < iters;) {
    if (!launch_persist_fire(d, fire, d_tab, ftol, dt_max, iters - k, d_persist, stream)) {
      cudaGetLastError();
      fail(SC_E_CUDA, "persistent FIRE kernel: cooperative launch failed");
      return false;
    }
    kernels += 1;
    if (!cuda_ok(cudaMemcpyAsync(h_pinned + 3, d_persist, sizeof(int), cudaMemcpyDeviceToHost,
                                 stream), "persist result") ||
        !cuda_ok(cudaStreamSynchronize(stream), "persist result"))
      return false;
    const int v = h_pinned[3];
    const int m = v >> 2, why = v & 3;
    if (m < 1 || m > iters - k || why == 3) {
      if (!check_status("persistent FIRE")) return false;
      fail(SC_E_STATE, "persistent FIRE kernel returned %d", v);
      return false;
    }
    k += m;
    if (why == 2) break;  // every system has converged
    if (why == 1) {
      launch_rb_worklist(d, d_tab, 0, stream);
      launch_mx_materialize(d, d_tab, 0, false, stream);
      launch_rebuild(d, true, d_tab, 0, stream, true);
      kernels += 14;
    }
  }
  return true;
}

// FIRE on every system until max |F| < ftol (or max_iter iterations); the host
// looks at the per-system state only between chunks of iterations.
int Handle::fire_minimize(double ftol, int max_iter, double dt0, double dt_max, int* iters,
                          double* fmax_out, int* done_out) {
  if (!(ftol > 0) || max_iter < 0 || !(dt0 > 0) || !(dt_max >= dt0)) {
    fail(SC_E_ARG, "fire: need ftol > 0, max_iter >= 0, 0 < dt0 <= dt_max");
    return SC_E_ARG;
  }
  cudaSetDevice(device);
  if (!ensure_fire()) return last_status;
  std::vector<StepScalars> rows(nsys);
  for (int s = 0; s < nsys; s++) rows[s] = row_current(s);
  if (!upload_table(rows)) return last_status;
  launch_fire_reset(d, fire, dt0, stream);
  std::vector<FireSys> hsys(nsys);
  const bool mixed = prec == PREC_MIXED;
  const bool persist = opt.persist_steps && mixed && d.pass_kind == 0 && d_persist;
  int it = 0;
  bool all_done = false;
  while (it < max_iter && !all_done) {
    int chunk = std::min(kFireChunk, max_iter - it);
    if (persist) {
      if (!run_persist_fire(chunk, ftol, dt_max)) return last_status;
    } else if (!(opt.use_graphs && chunk == kFireChunk && run_fire_graph(chunk, ftol, dt_max))) {
      for (int k = 0; k < chunk; k++) enqueue_fire_iteration(ftol, dt_max);
    }
    it += chunk;
    if (!cuda_ok(cudaGetLastError(), "fire launch") ||
        !cuda_ok(cudaMemcpyAsync(hsys.data(), fire.sys, nsys * sizeof(FireSys),
                                 cudaMemcpyDeviceToHost, stream), "fire state") ||
        !check_status("fire"))
      return last_status;
    all_done = true;
    for (auto& q : hsys) all_done = all_done && q.done;
  }
  pred_valid = false;
  forces_valid = false;
  if (mixed) fp64_valid = false;
  int max_it = 0;
  fire_iters.assign(nsys, 0);
  for (int s = 0; s < nsys; s++) {
    fire_iters[s] = hsys[s].iters;
    if (fmax_out) fmax_out[s] = hsys[s].fmax;
    if (done_out) done_out[s] = hsys[s].done;
    max_it = std::max(max_it, hsys[s].iters);
  }
  if (iters) *iters = max_it;
  return all_done ? SC_OK : SC_E_NOCONV;
}

// ---- conjugate gradient (cjpr_relax_2p, src/cuda/2point_dynamics.cu:4233-4296) ----

bool Handle::ensure_cg() {
  if (!ensure_fire()) return false;  // the search direction lives in the minimiser arrays
  if (cg.sys) return true;
  double *x0 = nullptr, *y0 = nullptr, *p0 = nullptr, *part = nullptr;
  CgSys* sys = nullptr;
  int* searching = nullptr;
  if (!dalloc(&x0, ntot, "cg f0x") || !dalloc(&y0, ntot, "cg f0y") ||
      !dalloc(&p0, ntot, "cg f0p") || !dalloc(&sys, nsys, "cg sys") ||
      !dalloc(&part, 3 * (size_t)d.npchunks, "cg partials") ||
      !dalloc(&searching, 1, "cg flag"))
    return false;
  cg.sys = sys;
  cg.part = part;
  cg.searching = searching;
  cg.max_probes = opt.cg_max_probes > 0 ? opt.cg_max_probes : kCgMaxProbes;
  d.cg0x = x0;  // the rebuild permutes the previous forces from now on
  d.cg0y = y0;
  d.cg0p = p0;
  invalidate_graph();
  return true;
}

// forces and energy at the state, then the start of each system's iteration
void Handle::enqueue_cg_head(int max_iter, unsigned long long search, cudaStream_t st) {
  cudaStream_t keep = stream;
  stream = st;
  launch_pass(PASS_FORCE, true, 0);
  launch_se_reduce(d, st);
  launch_cg_begin(d, cg, max_iter, search, st);
  kernels += 5;
  stream = keep;
}

// one line-search probe of every searching system: x_t, E(x_t), the next transition
void Handle::enqueue_cg_probe(unsigned long long search, cudaStream_t st) {
  cudaStream_t keep = stream;
  stream = st;
  launch_cg_probe(d, cg, st);
  launch_pass(PASS_ENERGY_T, true, 0);
  launch_se_reduce(d, st);
  launch_cg_search(d, cg, search, st);
  kernels += 4;
  stream = keep;
}

// the chosen move (with the rebuild request through `cond` inside a graph)
void Handle::enqueue_cg_move(unsigned long long cond, cudaStream_t st) {
  Dev dd = d;
  dd.cond = cond;
  launch_cg_move(dd, cg, st);
  kernels += 2;
}

// kCgChunk iterations as one graph: per iteration the head, the line search in a
// WHILE node (switched on by the head, off by the search when no system probes
// again), the move, and the rebuild chain in an IF node the move switches on.
bool Handle::run_cg_graph(int max_iter) {
  if (!use_conditional) return false;
  if (!cg_exec || cg_key_iter != max_iter) {
    if (cg_exec) cudaGraphExecDestroy(cg_exec);
    cg_exec = nullptr;
    cg_key_iter = -1;
    if (!stream2 && !cuda_ok(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking), "stream"))
      return false;
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    long long k0 = kernels;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < kCgChunk && e == cudaSuccess; k++) {
      cudaGraphConditionalHandle hs, hr;
      e = new_cond_handle(&hs, 0);
      if (e != cudaSuccess) break;
      enqueue_cg_head(max_iter, hs, stream);
      e = add_cond_body(
          hs, [&](cudaStream_t st2) { enqueue_cg_probe(hs, st2); return 4; },
          cudaGraphCondTypeWhile);
      if (e != cudaSuccess) break;
      e = new_cond_handle(&hr, 0);
      if (e != cudaSuccess) break;
      enqueue_cg_move(hr, stream);
      e = add_cond_body(hr, [&](cudaStream_t st2) {
        launch_rebuild(d, false, d_tab, 0, st2);
        return 12;
      });
    }
    kernels = k0;
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(stream, &g);
    cudaGraphExec_t ex = nullptr;
    if (e == cudaSuccess && e2 == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    cg_exec = ex;
    cg_key_iter = max_iter;
  }
  kernels += 7LL * kCgChunk;
  return cuda_ok(cudaGraphLaunch(cg_exec, stream), "cg graph launch");
}

// The same iterations launched from the host, which reads the "searching" word
// after every probe (the reference's host-driven line search).
bool Handle::run_cg_eager(int max_iter) {
  for (int k = 0; k < kCgChunk; k++) {
    if (!cuda_ok(cudaMemsetAsync(cg.searching, 0, sizeof(int), stream), "cg flag")) return false;
    enqueue_cg_head(max_iter, 0, stream);
    // the device ends every search within max_probes probes; this bound only
    // guards the host against a device state that never clears the word
    for (int probe = 0;; probe++) {
      if (probe > cg.max_probes + 8) {
        fail(SC_E_NOCONV, "cg: a line search did not end within its probe cap");
        return false;
      }
      int searching = 0;
      if (!cuda_ok(cudaMemcpyAsync(h_pinned + 2, cg.searching, sizeof(int),
                                   cudaMemcpyDeviceToHost, stream), "cg flag") ||
          !cuda_ok(cudaStreamSynchronize(stream), "cg flag"))
        return false;
      searching = h_pinned[2];
      if (!searching) break;
      enqueue_cg_probe(0, stream);
    }
    enqueue_cg_move(0, stream);
    launch_rebuild(d, false, d_tab, 0, stream);
    kernels += 12;
  }
  return cuda_ok(cudaGetLastError(), "cg launch");
}

// Conjugate gradient on every system until each stops by the reference's rules
// (zero force, three equal energies, no lower energy along any direction) or has
// taken max_iter iterations; the host reads the per-system state between chunks.
int Handle::cg_minimize(int max_iter, int* iters, double* energy, int* reason) {
  if (max_iter < 0) {
    fail(SC_E_ARG, "cg: max_iter must be >= 0");
    return SC_E_ARG;
  }
  if (prec != PREC_FP64) {
    fail(SC_E_STATE, "cg: the conjugate-gradient minimiser runs in the FP64 form");
    return SC_E_STATE;
  }
  cudaSetDevice(device);
  if (!ensure_cg()) return last_status;
  // rows at fixed gamma and box; the probes' energy pass reads the corrector fields
  std::vector<StepScalars> rows(nsys);
  for (int s = 0; s < nsys; s++) {
    StepScalars t = row_current(s);
    t.gamma_c = t.gamma_p;
    t.Lx_c = t.Lx_p;
    t.Ly_c = t.Ly_p;
    t.W_c = t.W_p;
    t.H_c = t.H_p;
    rows[s] = t;
  }
  if (!upload_table(rows)) return last_status;
  launch_cg_reset(d, cg, stream);
  std::vector<CgSys> hsys(nsys);
  bool all_done = false;
  while (!all_done) {
    if (!(opt.use_graphs && run_cg_graph(max_iter)) && !run_cg_eager(max_iter))
      return last_status;
    if (!cuda_ok(cudaGetLastError(), "cg launch") ||
        !cuda_ok(cudaMemcpyAsync(hsys.data(), cg.sys, nsys * sizeof(CgSys),
                                 cudaMemcpyDeviceToHost, stream), "cg state") ||
        !check_status("cg"))
      return last_status;
    all_done = true;
    for (auto& q : hsys) all_done = all_done && q.done;
  }
  pred_valid = false;
  forces_valid = false;
  bool capped = false, probes = false;
  for (int s = 0; s < nsys; s++) {
    if (iters) iters[s] = hsys[s].iters;
    if (energy) energy[s] = hsys[s].E0;
    if (reason) reason[s] = hsys[s].reason;
    capped = capped || hsys[s].reason == CG_MAX_ITER;
    probes = probes || hsys[s].reason == CG_PROBES;
  }
  if (probes) {
    fail(SC_E_NOCONV, "cg: a line search reached its probe cap (reason SC_CG_PROBES)");
    return SC_E_NOCONV;
  }
  return capped ? SC_E_NOCONV : SC_OK;
}

// Box and positions of each system scaled by factor[s] (1 leaves it alone), in y
// alone with y_only (resize_y_coords_2p).
int Handle::affine_scale(const std::vector<double>& factor, bool y_only) {
  cudaSetDevice(device);
  if (!materialize()) return last_status;
  std::vector<double> fxy(2 * (size_t)nsys);
  for (int s = 0; s < nsys; s++) {
    fxy[2 * s] = y_only ? 1.0 : factor[s];
    fxy[2 * s + 1] = factor[s];
  }
  double* dfac = nullptr;
  if (!dalloc(&dfac, 2 * (size_t)nsys, "factors")) return last_status;
  bool ok = cuda_ok(cudaMemcpyAsync(dfac, fxy.data(), 2 * nsys * sizeof(double),
                                    cudaMemcpyHostToDevice, stream), "factors");
  if (ok) launch_affine(d, dfac, stream);
  ok = ok && cuda_ok(cudaStreamSynchronize(stream), "affine");
  dfree(dfac);
  if (!ok) return last_status;
  bool regrid = false;
  for (int s = 0; s < nsys; s++) {
    if (factor[s] == 1.0) continue;
    HostSys& h = hs[s];
    const double old_x = h.Lx, old_y = h.Ly;
    if (!y_only) h.Lx *= factor[s];
    h.Ly *= factor[s];
    h.packing *= y_only ? old_y / h.Ly : (old_x / h.Lx) * (old_x / h.Lx);
    int r = h.rows, c = h.cols;
    h.configure(false);
    if (h.rows != r || h.cols != c) regrid = true;
  }
  if (regrid && !layout_cells()) return last_status;
  return rebuild_all() && check_status("affine scale") ? SC_OK : last_status;
}

// Reverses the shear direction of the selected systems (flip_shear_direction,
// src/cuda/find_neighbors.cu:563-581): positions reflected about the box's y axis,
// angles negated, gamma negated, then the cell lists rebuilt.
int Handle::flip_shear(const std::vector<char>& sel) {
  cudaSetDevice(device);
  if (!materialize()) return last_status;
  std::vector<double> lx(nsys, 0.0);
  for (int s = 0; s < nsys; s++)
    if (sel[s]) lx[s] = hs[s].Lx;
  double* dl = nullptr;
  if (!dalloc(&dl, nsys, "flip")) return last_status;
  bool ok = cuda_ok(cudaMemcpyAsync(dl, lx.data(), nsys * sizeof(double), cudaMemcpyHostToDevice,
                                    stream), "flip");
  if (ok) launch_reflect(d, dl, stream);
  ok = ok && cuda_ok(cudaStreamSynchronize(stream), "flip");
  dfree(dl);
  if (!ok) return last_status;
  for (int s = 0; s < nsys; s++)
    if (sel[s]) hs[s].gamma = -hs[s].gamma;
  return rebuild_all() && check_status("flip shear") ? SC_OK : last_status;
}

// Turns the selected systems to the frame in which their sheared cell is upright
// (rotate_by_gamma, src/cuda/find_neighbors.cu:626-645): Lx' = Ly sqrt(1 + g^2),
// Ly' = Lx / sqrt(1 + g^2), gamma -> -gamma, positions and angles mapped by
// k_rotate; the cell grid is configured for the new box and the lists rebuilt.
int Handle::rotate_shear(const std::vector<char>& sel) {
  cudaSetDevice(device);
  if (!materialize()) return last_status;
  std::vector<double> q(4 * (size_t)nsys, 0.0);
  for (int s = 0; s < nsys; s++)
    if (sel[s]) {
      HostSys& h = hs[s];
      const double lx = h.Lx, ly = h.Ly;
      h.Lx = ly * std::sqrt(1 + h.gamma * h.gamma);
      h.Ly = lx / std::sqrt(1 + h.gamma * h.gamma);
      q[4 * s] = h.gamma;
      q[4 * s + 1] = h.Lx;
      q[4 * s + 2] = h.Ly;
      q[4 * s + 3] = 1.0;
      h.gamma = -h.gamma;
      h.configure(false);
    }
  double* dq = nullptr;
  if (!dalloc(&dq, q.size(), "rotate")) return last_status;
  bool ok = cuda_ok(cudaMemcpyAsync(dq, q.data(), q.size() * sizeof(double),
                                    cudaMemcpyHostToDevice, stream), "rotate");
  if (ok) launch_rotate(d, dq, stream);
  ok = ok && cuda_ok(cudaStreamSynchronize(stream), "rotate");
  dfree(dq);
  if (!ok) return last_status;
  return layout_cells() && rebuild_all() && check_status("rotate shear") ? SC_OK : last_status;
}

// run_strain(dGammaMax), src/cuda/strain_dynamics.cu:1097-1108: shear without
// setting gamma back until gamma >= gamma_max (no output), on a cell grid wide
// enough for that gamma (reconfigure_cells(dGammaMax), src/cuda/spherocyl_box.cpp:
// 46-67); the grid keeps that width afterwards.  One system per handle.
int Handle::strain_to_gamma(double gamma_max, long* steps_out) {
  if (nsys != 1) {
    fail(SC_E_ARG, "sc_strain_to_gamma: one system per handle");
    return SC_E_ARG;
  }
  HostSys& S = hs[0];
  if (!(S.strain_rate > 0) || !(S.step > 0) || !std::isfinite(gamma_max)) {
    fail(SC_E_ARG, "sc_strain_to_gamma: needs a positive strain rate and step");
    return SC_E_ARG;
  }
  // the steps the loop takes, with the host mirror's own accumulation
  long k = 0;
  for (double g = S.gamma; g < gamma_max; g += S.strain_rate * S.step)
    if (++k > (1L << 31)) {
      fail(SC_E_ARG, "sc_strain_to_gamma: too many steps");
      return SC_E_ARG;
    }
  if (steps_out) *steps_out = k;
  if (k == 0) return SC_OK;
  cudaSetDevice(device);
  const double w = 2 * std::sqrt(gamma_max * gamma_max + 1);
  if (w > S.wfac) {
    if (!materialize()) return last_status;
    S.wfac = w;
    S.configure(false);
    if (!layout_cells() || !rebuild_all()) return last_status;
  }
  S.setback = false;
  int rc = SC_OK;
  for (long done = 0; done < k && rc == SC_OK;) {
    const int chunk = (int)std::min<long>(k - done, 1L << 20);
    rc = run_steps(KIND_STRAIN, 0, chunk, 0, nullptr);
    done += chunk;
  }
  hs[0].setback = true;
  return rc;
}

// Quasistatic compression to jamming: affine steps of dphi in packing fraction,
// each followed by a FIRE minimisation; a system stops once its energy per
// particle after minimisation exceeds e_jam (compress_qs2p / find_jam_2p,
// src/cuda/2point_dynamics.cu:4299-4344, 4582-4606, with FIRE for the relaxation).
int Handle::quasistatic(double dphi, double ftol, double e_jam, int max_inc, int max_iter,
                        double* phi_jam, int* n_inc) {
  if (!(dphi > 0) || !(e_jam >= 0) || max_inc < 0) {
    fail(SC_E_ARG, "quasistatic: need dphi > 0, e_jam >= 0, max_inc >= 0");
    return SC_E_ARG;
  }
  std::vector<char> jammed(nsys, 0);
  std::vector<double> se(5 * (size_t)nsys);
  int inc = 0;
  int rc = fire_minimize(ftol, max_iter, 1e-2, 0.2, nullptr, nullptr, nullptr);
  if (rc && rc != SC_E_NOCONV) return rc;
  for (inc = 0; inc < max_inc; inc++) {
    std::vector<double> f(nsys, 1.0);
    bool any = false;
    for (int s = 0; s < nsys; s++)
      if (!jammed[s]) {
        f[s] = std::sqrt(hs[s].packing / (hs[s].packing + dphi));
        any = true;
      }
    if (!any) break;
    if ((rc = affine_scale(f))) return rc;
    rc = fire_minimize(ftol, max_iter, 1e-2, 0.2, nullptr, nullptr, nullptr);
    if (rc && rc != SC_E_NOCONV) return rc;
    if ((rc = calc(true, se.data()))) return rc;
    for (int s = 0; s < nsys; s++)
      if (!jammed[s] && se[5 * s] > e_jam) {
        jammed[s] = 1;
        if (phi_jam) phi_jam[s] = hs[s].packing;
      }
  }
  for (int s = 0; s < nsys; s++)
    if (!jammed[s] && phi_jam) phi_jam[s] = -hs[s].packing;  // not jammed: negative
  if (n_inc) *n_inc = inc;
  return SC_OK;
}

// Jamming point by bisection on the energy (find_jam_2p with resize_to_energy_2p,
// src/cuda/2point_dynamics.cu:4582-4606, 4393-4456), per system: a phase
// compresses while E/N < e_jam (expands while E/N > e_jam) by affine length steps
// of 1 - step (1 / (1 - step)), minimising after each and growing the step by 1.1 per
// step; once the energy has crossed e_jam the next phase starts the other way with
// half the last step, until the step falls below min_step.  e_jam is an energy per
// particle, or with per_area the reference's measure (calc_fe_2p's energy per unit
// area, E/N x N / 2LxLy); on_step sees each resize's stress/energy; cg_relax relaxes
// with the conjugate gradient (cjpr_relax_2p) instead of FIRE; y_only resizes Ly and
// the y coordinates alone (y_compress_energy_2p with y_resize_step_2p).
int Handle::find_jam(double e_jam, double step0, double min_step, double ftol, int max_iter,
                     int max_steps, double* phi_jam, int* steps_out,
                     const std::function<int(int, const double*)>& on_step, bool cg_relax,
                     bool per_area, bool y_only) {
  if (!(e_jam > 0) || !(step0 > 0) || !(min_step > 0) || max_steps < 0) {
    fail(SC_E_ARG, "find_jam: need e_jam > 0, step > 0, min_step > 0, max_steps >= 0");
    return SC_E_ARG;
  }
  struct Phase {
    int dir = 0;          // +1 compress, -1 expand, 0 finished
    double step = 0;      // step of this phase's first resize
    double next = 0;      // step of the next resize
    int k = 0;            // resizes made in this phase
  };
  std::vector<Phase> ph(nsys);
  std::vector<double> se(5 * (size_t)nsys);
  // cjpr_relax_2p (the reference's relaxation here) or FIRE to ftol
  auto relax = [&]() {
    return cg_relax ? cg_minimize(max_iter, nullptr, nullptr, nullptr)
                    : fire_minimize(ftol, max_iter, 1e-2, 0.2, nullptr, nullptr, nullptr);
  };
  // the compared energy: per particle, or calc_fe_2p's energy per unit area, which
  // sums (1 - d/sigma)^2 / (4 Lx Ly) per contact side against (1 - d/sigma)^2 / 2N
  auto energy = [&](int s) {
    const HostSys& h = hs[s];
    return per_area ? se[5 * s] * (double)h.n / (2.0 * h.Lx * h.Ly) : se[5 * s];
  };
  int rc = relax();
  if (rc && rc != SC_E_NOCONV) return rc;
  if ((rc = calc(true, se.data()))) return rc;
  auto start_phase = [&](int s, double step) {
    Phase& q = ph[s];
    const double e = energy(s);
    // an energy exactly at e_jam makes every later phase empty (only the step
    // shrinks), so the system is finished where it is
    q.dir = e < e_jam ? 1 : (e > e_jam ? -1 : 0);
    q.step = q.next = step;
    q.k = 0;
  };
  for (int s = 0; s < nsys; s++) start_phase(s, step0);
  if (!(step0 > min_step))
    for (auto& q : ph) q.dir = 0;
  int steps = 0;
  for (; steps < max_steps; steps++) {
    std::vector<double> f(nsys, 1.0);
    bool any = false;
    for (int s = 0; s < nsys; s++)
      if (ph[s].dir != 0) {
        // the step grows by 1.1 per resize while e_jam is not crossed; at 1 the
        // length factor would reach zero (the reference has no such check)
        if (!(ph[s].next < 1.0)) {
          fail(SC_E_NOCONV, "find_jam: the resize step reached 1 before the energy crossed e_jam");
          return SC_E_NOCONV;
        }
        // resize_step_2p (src/cuda/2point_dynamics.cu:1187-1195): lengths x (1 - step)
        // to compress, / (1 - step) to expand
        f[s] = ph[s].dir > 0 ? 1.0 - ph[s].next : 1.0 / (1.0 - ph[s].next);
        any = true;
      }
    if (!any) break;
    if ((rc = affine_scale(f, y_only))) return rc;
    rc = relax();
    if (rc && rc != SC_E_NOCONV) return rc;
    if ((rc = calc(true, se.data()))) return rc;
    // each resize's output (resize_to_energy_2p writes a line and a file per step)
    if (on_step && (rc = on_step(steps + 1, se.data()))) return rc;
    for (int s = 0; s < nsys; s++) {
      Phase& q = ph[s];
      if (q.dir == 0) continue;
      q.k += 1;
      q.next *= 1.1;
      const double e = energy(s);
      const bool crossed = q.dir > 0 ? !(e < e_jam) : !(e > e_jam);
      if (!crossed) continue;
      // find_jam_2p: dResizeStep * 1.1^(steps in the phase - 1) / 2
      const double step = q.step * std::pow(1.1, q.k - 1) / 2;
      if (!(step > min_step)) {
        q.dir = 0;
        continue;
      }
      start_phase(s, step);
    }
  }
  for (int s = 0; s < nsys; s++)
    if (phi_jam) phi_jam[s] = ph[s].dir == 0 ? hs[s].packing : -hs[s].packing;
  if (steps_out) *steps_out = steps;
  return SC_OK;
}

}  // namespace sc
