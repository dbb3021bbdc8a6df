// sc_host.hpp -- the handle behind the C ABI (host side only).
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>
#include <vector>

#include "../../include/spherocyl.h"
#include "sc_internal.hpp"

namespace sc {

// Host mirror of one system: the scalars the reference's SpherocylBox keeps
// (src/cpp/spherocyl_box.h:29-61), advanced with the reference's arithmetic.
struct HostSys {
  int n = 0, p0 = 0;
  double Lx = 0, Ly = 0;
  double gamma = 0, gamma_total = 0;
  double strain_rate = 0, resize_rate = 0;
  double step = 0.05;  // set_defaults, src/cpp/spherocyl_box.cpp:24
  double pad = 0;
  double Rmax = 0, Amax = 0;
  double packing = 0;
  int rows = 1, cols = 1;
  int ntx = 1, nty = 1;  // tiles across and down (the tile pass's cell numbering)
  int c0 = 0, chunk0 = 0, nchunks = 0;
  // cell width over R_max + A_max (configure_cells, src/cpp/spherocyl_box.cpp:225:
  // 2.24, enough for |gamma| <= 1/2; 2 sqrt(1 + gamma^2) for a run to larger gamma,
  // src/cuda/spherocyl_box.cpp:132-144) and whether gamma is set back at 1/2
  double wfac = 2.24;
  bool setback = true;

  void configure(bool set_pad);
  bool grid_changes_xy(double Lx_now, double Ly_now) const;
};

// kinds of Heun step the step table describes
enum StepKind { KIND_STRAIN = 0, KIND_RESIZE = 1, KIND_PURE = 2 };

struct GraphKey {
  bool resize = false;
  int nsteps = 0, se_every = -1;
  int prec = -1;
  bool operator==(const GraphKey& o) const {
    return resize == o.resize && nsteps == o.nsteps && se_every == o.se_every && prec == o.prec;
  }
};

// The memory pool of a device that all handles on it allocate from (nullptr where
// the device has no stream-ordered pools).  Freed blocks stay in the pool for the
// next handle until sc_trim_memory releases them.
cudaMemPool_t device_pool(int device);

struct Handle {
  static constexpr int kChunk = 100;  // steps per table upload / captured graph
  static constexpr int kFireChunk = 50;  // FIRE iterations between host checks

  sc_options opt{};
  int device = -1;
  int prec = PREC_FP64;
  int block = 128;
  int nsys = 0, ntot = 0;
  std::vector<HostSys> hs;
  std::vector<double> h_R, h_A;  // particle radii and half shafts, input order (on demand)
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Dev d{};
  std::vector<void*> allocs;
  int cell_cap = 0, chunk_cap = 0, tile_cap = 0;
  const int* pass_skip = nullptr;  // Dev::skip of the force passes being enqueued
  int* d_persist = nullptr;        // result word of the persistent step kernel
  StepScalars* d_tab = nullptr;
  int tab_cap = 0;
  std::vector<StepScalars> h_tab;
  double* d_se_hist = nullptr;
  double* d_out3 = nullptr;  // [3 * ntot] output staging in the caller's particle order
  int se_hist_cap = 0;
  int* h_pinned = nullptr;  // status word + scratch for small reads
  bool pred_valid = false;  // predictor copy consistent with the state
  int pred_kind = 0;        // 1 strain, 2 shrink, 3 grow, 4 pure shear
  bool fp64_valid = true;   // mixed form: FP64 copy of the state is current
  bool forces_valid = false;// mixed form: fx/fy/tau hold the forces of the state
  long long steps = 0, rebuilds = 0;
  int dev_status = 0;
  long long dev_rebuilds = 0;  // rebuild chains the device executed
  long long kernels = 0;       // kernels launched (eagerly or inside graphs)
  long long graph_kernels = 0; // kernels in the last captured graph
  long long chunk_kernels = 0; // kernels in the chunk graph (graph_exec)
  int last_status = SC_OK;
  std::string err;
  // CUDA graph of one chunk of steps
  cudaGraphExec_t graph_exec = nullptr;
  GraphKey graph_key{};
  // Chunks whose length is a multiple of kGraphSteps run as sub-chunk graphs of
  // kGraphSteps steps, which read their rows from a window of the step table (d_win,
  // refilled before each launch) and leave their records in d_win_se: a graph 10x
  // shorter to capture and instantiate, reused for every sub-chunk with the same step
  // kind and the same steps recording stress/energy (se_mask).
  static constexpr int kGraphSteps = 10;
  struct SubGraph {
    bool resize;
    unsigned se_mask;
    int prec;
    cudaGraphExec_t exec;
    long long kernels;
  };
  std::vector<SubGraph> sub_graphs;
  StepScalars* d_win = nullptr;
  double* d_win_se = nullptr;
  cudaStream_t stream2 = nullptr;  // captures the conditional rebuild bodies
  bool use_conditional = true;     // conditional graph nodes available
  bool graph_conditional = false;  // the current graph uses them
  long long body_kernels = 0;      // kernels in one rebuild body
  // CUDA graph of one chunk of FIRE iterations (same conditional rebuild node)
  cudaGraphExec_t fire_exec = nullptr;
  int fire_key_iters = 0;
  double fire_key_ftol = 0, fire_key_dtmax = 0;
  long long fire_graph_kernels = 0;
  // profiling: per-pass events
  struct Mark {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<cudaEvent_t> ev_pool;
  int ev_used = 0;
  std::vector<Mark> ev_marks;
  double pass_ms[3] = {0, 0, 0};
  long long pass_n[3] = {0, 0, 0};

  ~Handle();
  void fail(int code, const char* fmt, ...);
  bool cuda_ok(cudaError_t e, const char* what);
  bool use_pool = false;  // device memory comes from the device's cached pool
  template <class T>
  bool dalloc(T** p, size_t count, const char* what) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = use_pool ? cudaMallocFromPoolAsync((void**)p, count * sizeof(T),
                                                       device_pool(device), stream)
                             : cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
      fail(SC_E_NOMEM, "cudaMalloc %s (%zu bytes): %s", what, count * sizeof(T),
           cudaGetErrorString(e));
      *p = nullptr;
      return false;
    }
    allocs.push_back((void*)*p);
    return true;
  }
  void dfree(void* p);

  StepScalars row_current(int s) const;
  bool layout_cells();
  bool ensure_table(int rows);
  bool upload_table(const std::vector<StepScalars>& rows);
  bool ensure_se_hist(int nrec);
  bool check_status(const char* where);
  bool rebuild_all();
  void launch_pass(int mode, bool se, int row, bool fast = false);
  cudaEvent_t next_event();
  void timed(int kind, bool on, const std::function<void()>& f);
  void collect_times();
  void enqueue_step(bool resize, int k, bool se, bool prof);
  void enqueue_corr(bool resize, int k, bool prof);
  int enqueue_rebuild_body(bool resize, int k, bool prof, cudaStream_t st);
  void enqueue_pred(bool resize, int k, bool se, bool prof);
  cudaError_t capture_rebuild_node(int row, const std::function<int(cudaStream_t)>& body);
  cudaError_t new_cond_handle(cudaGraphConditionalHandle* h);
  cudaError_t add_cond_body(cudaGraphConditionalHandle h,
                            const std::function<int(cudaStream_t)>& body,
                            cudaGraphConditionalNodeType type = cudaGraphCondTypeIf);
  cudaError_t new_cond_handle(cudaGraphConditionalHandle* h, unsigned int dflt);
  unsigned long long step_cond = 0;  // rebuild node of the step being captured
  bool capture_conditional(bool resize, int nsteps, const std::vector<char>& se,
                           cudaGraph_t* out);
  bool instantiate_steps(bool resize, int nsteps, const std::vector<char>& se,
                         cudaGraphExec_t* exec, long long* nkernels);
  bool run_subgraphs(bool resize, int nsteps, int se_every);
  void enqueue_se_record(int rec);
  void invalidate_graph();
  bool run_graph(bool resize, int nsteps, int se_every);
  SubGraph* subgraph(bool resize, unsigned mask);
  void invalidate_table_graphs();
  bool run_persist(int nk, int done, int se_every);
  bool run_persist_fire(int iters, double ftol, double dt_max);
  bool ensure_host_shapes();  // fills h_R, h_A from the device on first use
  std::vector<int> fire_iters;  // per-system iterations of the last FIRE run

  int run_steps(int kind, int shrink, int nsteps, int se_every, double* se_out);
  int calc(bool se, double* se_out);
  bool materialize();
  bool read_unsorted(bool forces, double* a, double* b, double* c);
  int gd_minimize(int max_steps, double e_min, int* steps_taken, double* e_final);
  int gd_step(const double* se_now, double e_min);
  // FIRE minimiser and quasistatic compression
  FireState fire{};
  bool ensure_fire();
  void enqueue_fire_iteration(double ftol, double dt_max);
  bool run_fire_graph(int iters, double ftol, double dt_max);
  int fire_minimize(double ftol, int max_iter, double dt0, double dt_max, int* iters,
                    double* fmax_out, int* done_out);
  int affine_scale(const std::vector<double>& factor, bool y_only = false);
  // Polak-Ribiere conjugate gradient with the reference's line search
  CgState cg{};
  static constexpr int kCgChunk = 10;  // iterations per captured graph
  cudaGraphExec_t cg_exec = nullptr;
  int cg_key_iter = -1;
  bool ensure_cg();
  void enqueue_cg_head(int max_iter, unsigned long long search, cudaStream_t st);
  void enqueue_cg_probe(unsigned long long search, cudaStream_t st);
  void enqueue_cg_move(unsigned long long cond, cudaStream_t st);
  bool run_cg_graph(int max_iter);
  bool run_cg_eager(int max_iter);
  int cg_minimize(int max_iter, int* iters, double* energy, int* reason);
  int flip_shear(const std::vector<char>& sel);
  int rotate_shear(const std::vector<char>& sel);
  int strain_to_gamma(double gamma_max, long* steps);
  int quasistatic(double dphi, double ftol, double e_jam, int max_inc, int max_iter,
                  double* phi_jam, int* n_inc);
  int find_jam(double e_jam, double step0, double min_step, double ftol, int max_iter,
               int max_steps, double* phi_jam, int* steps_out,
               const std::function<int(int, const double*)>& on_step = nullptr,
               bool cg_relax = false, bool per_area = false, bool y_only = false);
};

// last error of calls made without a handle (creation, file reading)
extern thread_local std::string g_noh_error;

}  // namespace sc

struct sc_handle {
  sc::Handle h;
};
