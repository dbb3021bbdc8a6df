// sc_internal.hpp -- data layout shared by the host runtime and the sm_103a kernels.
//
// Layout in HBM (all arrays indexed by "slot": particles sorted by cell, systems
// contiguous; system s owns slots [p0, p0+n) and global cells [c0, c0+cols*rows)):
//   xy  double2  centre position in sheared (Lees-Edwards) coordinates
//   ph  double   orientation angle
//   ra  double2  (R, A): radius and half shaft length
//   irc double2  (I, RC): rotational drag factor and isolated-rotation coefficient
//   id  int      particle index within its system (the reference's particle order)
//   cell int     global cell index assigned at the last rebuild
// plus per-pass working arrays (predictor copy, Heun velocities, forces, moved
// distance) and, for the mixed form, an FP32 geometry record per particle.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sc {

enum Precision { PREC_FP64 = 0, PREC_MIXED = 1 };
enum StressMode { STRESS_COMPAT = 0, STRESS_VIRIAL = 1 };

#ifdef __CUDACC__
#define SC_HDI __host__ __device__ __forceinline__
#else
#define SC_HDI inline
#endif

// Per-system constants of the current cell grid; changed only by the host.
struct SysGeom {
  int n, p0;           // particle count and first slot
  int c0, cols, rows;  // first global cell and grid dimensions
  int chunk0, nchunks; // cell-scan chunks owned by the system
  int ntx, nty;        // tiles across and down (cell numbering, see cell_local)
  int pch0;            // first particle-reduction chunk (kSeChunk particles each)
  double pad;          // neighbour padding (configure_cells auto-value applied)
  double inv_n;        // 1/n, energy normalisation
  float smax;          // largest R_i + A_i + R_j + A_j of the system
  float fpad;          // pad in FP32
};

// Cell numbering of a system.  The grid is cut into ntx x nty tiles of nearly
// equal size (tile k along a dimension of n cells covers [k n / nt, (k+1) n / nt));
// cells are numbered tile by tile (tiles row-major), row-major inside a tile.  The
// particles of a tile then occupy one contiguous range of slots, which the tile
// force pass stages in shared memory.  With one tile (ntx = nty = 1, the FP64
// form) this is the reference's col + row * cols.
// (n < 65536 cells a side, so the products fit 32 unsigned bits)
SC_HDI int tile_lo(int k, int n, int nt) { return (int)(((unsigned)k * (unsigned)n) / (unsigned)nt); }
SC_HDI int tile_of(int c, int n, int nt) {
  if (nt == 1) return 0;
  int k = (int)(((unsigned)c * (unsigned)nt) / (unsigned)n);
  if (k > nt - 1) k = nt - 1;
  while (k + 1 < nt && tile_lo(k + 1, n, nt) <= c) k++;
  while (k > 0 && tile_lo(k, n, nt) > c) k--;
  return k;
}
// local cell index (add c0 for the global one) of column col, row row
SC_HDI int cell_local(const SysGeom& g, int col, int row) {
  if (g.ntx == 1 && g.nty == 1) return row * g.cols + col;
  const int kx = tile_of(col, g.cols, g.ntx), ky = tile_of(row, g.rows, g.nty);
  const int x0 = tile_lo(kx, g.cols, g.ntx), x1 = tile_lo(kx + 1, g.cols, g.ntx);
  const int y0 = tile_lo(ky, g.rows, g.nty), y1 = tile_lo(ky + 1, g.rows, g.nty);
  return y0 * g.cols + (y1 - y0) * x0 + (row - y0) * (x1 - x0) + (col - x0);
}
// column and row of local cell lc
SC_HDI void cell_colrow(const SysGeom& g, int lc, int* col, int* row) {
  if (g.ntx == 1 && g.nty == 1) {
    *row = lc / g.cols;
    *col = lc - *row * g.cols;
    return;
  }
  const int ky = tile_of(lc / g.cols, g.rows, g.nty);
  const int y0 = tile_lo(ky, g.rows, g.nty), hy = tile_lo(ky + 1, g.rows, g.nty) - y0;
  const int off = lc - y0 * g.cols;
  const int kx = tile_of(off / hy, g.cols, g.ntx);
  const int x0 = tile_lo(kx, g.cols, g.ntx), wx = tile_lo(kx + 1, g.cols, g.ntx) - x0;
  const int o2 = off - hy * x0;
  *row = y0 + o2 / wx;
  *col = x0 + o2 % wx;
}

// Per-(step, system) scalars, computed on the host with the reference's own
// floating-point operations so that gamma and the box lengths are bit-identical
// to the reference's accumulation.  Row 0 of a table primes the first step
// (only the *_p fields are used); rows 1..K are the K steps.
struct StepScalars {
  double gamma_c;    // gamma of the corrector force pass (gamma_k + dt*rate)
  double gamma_p;    // gamma of the following pass (gamma_{k+1}, after any set-back)
  double Lx_c, Ly_c; // box of the corrector pass minimum image
  double Lx_p, Ly_p; // box after the step (predictor pass and the next corrector)
  double W_c, H_c;   // cell size matching Lx_c, Ly_c
  double W_p, H_p;   // cell size matching Lx_p, Ly_p
  double rate;       // strain rate
  double step;       // integration step
  double scale;      // resize factor pow(1-rate, dt)
  int mode;          // 0 none, 1 multiply by scale (shrink), 2 divide by scale (grow),
                     // 3 pure shear (x stretched and y compressed at the strain rate)
  int setback;       // set back gamma at the end of this step
  // FP32 copies for the mixed form (no FP64 arithmetic in its passes)
  float f_gamma_c, f_gamma_p, f_Wc, f_Hc, f_Wp, f_Hp, f_rate, f_step;
  // affine increment of one step, x <- x + g x: scale - 1 (mode 1) or 1/scale - 1
  // (mode 2) on both axes, +dt rate/2 on x and -dt rate/2 on y (mode 3), else 0.
  // Held as the increment, not as 1 + g, so that FP32 keeps its relative precision.
  float f_gx, f_gy;
};

// FIRE minimiser state of one system
struct FireSys {
  double dt, alpha;  // current time step and mixing parameter
  double c1, c2;     // mixing coefficients of the coming update: v <- c1 v + c2 F/m
  double fmax;       // largest |F_i| (or |tau_i|/sqrt(I_i)) at the last evaluation
  int npos, zero_v, done, iters;
};

struct FireState {
  double* vx;
  double* vy;
  double* vp;
  FireSys* sys;   // [nsys]
  double* part;   // [4 * npchunks] chunk partials
  int* done;      // [nsys] copy of sys[s].done for the force passes (Dev::skip)
};

// Conjugate-gradient minimiser state of one system (the reference's line-search
// energies h_pdLineEnergy[0..4], step bounds and the search position as data)
enum CgPhase { CG_IDLE = 0, CG_TOP = 1, CG_SECOND = 2, CG_HALVE = 3, CG_DOUBLE = 4,
               CG_FINAL = 5, CG_MOVE = 6 };
enum CgReason { CG_RUNNING = 0, CG_ZERO_FORCE = 1, CG_STALLED = 2, CG_STEP = 3,
                CG_MAX_ITER = 4, CG_PROBES = 5 };
constexpr int kCgMaxProbes = 256;  // default probe cap of one line search
struct CgSys {
  double E0, E1, E2;     // energies at 0, one step and two steps along D
  double Eh1, Eh2;       // iteration-start energies of the two iterations before
  double F2, beta;       // |F|^2 and the Polak-Ribiere beta of this iteration
  double norm;           // |F|_rms = sqrt(|F|^2 / 3N)
  double step, min_step, max_step;
  double t, tmin;        // position of the next probe; the chosen multiple of step
  int phase, attempt;    // CgPhase; 0 PR direction, 1 steepest descent, 2 sqrt-scaled
  int redirect;          // the next probe first sets D (1: F, 2: F/sqrt|F|)
  int done, reason, iters;
  int probes;            // energy probes of this iteration's line search
};

struct CgState {
  CgSys* sys;      // [nsys]
  double* part;    // [3 * npchunks] chunk partials of |F|^2, F.F0, |F0|^2
  int* searching;  // any system probing (for the host-driven loop)
  int max_probes;  // a line search that needs more probes ends the system (CG_PROBES)
};

// Device pointers handed to every kernel by value.
struct Dev {
  int ntot, nsys, ncells, nchunks, npchunks;
  int maxn;                 // neighbour-list capacity per particle (FP64 form)
  int stress_mode;
  int contact_model;        // 0 one contact point (src/cpp), 1 two points (src/cuda 2p)
  const SysGeom* geom;      // [nsys]
  const int* psys;          // [ntot] system of each slot
  const int* cell_sys;      // [ncells] system of each cell
  // state
  double2* xy;
  double* ph;
  double2* ra;
  double2* irc;
  int* id;
  int* cell;
  double2* nxy;             // (A cos phi, A sin phi) of the state positions
  // predictor copy
  double2* xy_t;
  double* ph_t;
  double2* nxy_t;
  // Heun velocities of the predictor, forces, moved distance
  double* v0x;
  double* v0y;
  double* v0p;
  double* fx;
  double* fy;
  double* tau;
  double2* moved;
  // mixed form (FP32 state relative to the cell centre, compensated):
  float4* rec;    // (x_local, y_local, A cos phi, A sin phi) of the state
  float4* rec_t;  // the same for the predictor copy
  float4* mc;     // (x compensation, y compensation, phi, phi compensation)
  float4* mv;     // (v0x, v0y, v0phi, predicted phi)
  float4* mm;     // (x, y displacement since the last rebuild, angle at it, unused)
  float4* pa;     // (R, A, particle index as int bits, 1/I)
  float* rcf;     // isolated-rotation coefficient RC
  float* rf;      // R in FP32: the only per-neighbour constant the force pass gathers
  int* cellp;     // local cell packed as col | row << 16
  float* gbuild;  // [nsys] gamma at which each system's list was built
  // cell lists
  int* cell_start;          // [ncells] first slot
  int* cell_count;          // [ncells]
  // neighbour list, column-major [k * ntot + slot]
  int* nbr;
  int* nbr_n;
  // mixed form: the same lists reordered for the force pass.  Within each window
  // of kOrderWindow slots, threads take the slots in order of increasing list
  // length, so a warp's lanes loop over lists of nearly equal length.
  int* ord;     // [ntot] position -> slot
  int* nbr_p;   // column-major [k * ntot + position]
  int* nbr_pn;  // [ntot] list length at each position (capped at maxn)
  // mixed form, tile force pass (pass_kind 1): each tile's pairs once.  The tile's
  // compute entries (owner-major) and read entries live in the slot range of its
  // particles times kTileEPP; a pair inside the tile is computed by its lower slot
  // and read back by the other partner from the pair results.
  unsigned* gbar;           // [2] grid barrier of the persistent step kernel (count, generation)
  const int* skip;          // [nsys] or null: force passes leave systems with skip[s] != 0
                            // alone (converged minimiser systems)
  int pass_kind;            // 0: one thread per particle over its full list, 1: tiles
  int ntiles;
  const int4* tiles;        // [ntiles] (system, first global cell, cells, 0)
  int4* tinfo;              // [ntiles] (first slot, particles, compute entries, read entries)
  unsigned short* t_own;    // [ntot * kTileEPP] owner (index in the tile) of each entry
  unsigned* t_pe;           // [ntot * kTileEPP] partner: kTileInt | index in the tile, or
                            // the slot; the cell offset code in the top 4 bits
  unsigned* t_rd;           // [ntot * kTileEPP] read entries: the compute entry of the pair
  int2* t_meta;             // [ntot] (compute offset | count << 24, read offset | count << 24)
  float4* t_pb;             // [ntot * kTileEPP] pair results of tiles too large for shared memory
  // rebuild scratch
  int* cell_tmp;
  int* rank;
  int* perm;
  int* chunk_sum;
  int* chunk_off;
  const int* chunk_sys;     // [nchunks] system of each chunk
  const int* chunk_c0;      // [nchunks] first global cell of each chunk
  const int* chunk_nc;      // [nchunks] cells in the chunk
  double2* s_xy;
  double* s_ph;
  double2* s_ra;
  double2* s_irc;
  int* s_id;
  int* s_cell;
  // stress/energy: per-slot contributions and per-chunk partials
  double* se_part;          // [5][ntot]
  double* se_chunk;         // [5][npchunks]
  double* se_sys;           // [5][nsys]
  const int* pchunk_sys;    // particle chunks for reductions
  const int* pchunk_p0;
  const int* pchunk_np;
  // flags
  double* fvx;              // FIRE velocities or CG directions (null until a
  double* fvy;              // minimiser is used); permuted with the particles by
  double* fvp;              // the rebuild
  double* cg0x;             // CG: the previous iteration's forces (null until CG is
  double* cg0y;             // used), permuted with the particles by the rebuild
  double* cg0p;
  int* flags;               // [nsys] bit0 moved-rebuild, bit1 forced rebuild
  int* istar;               // [nsys] lowest particle index that triggered a rebuild
  int* any;                 // [1] set when any system needs a rebuild
  int* work;                // [nsys] rebuild worklist: the flagged systems, ascending
  int* woff;                // [nsys + 1] first work item (slot) of each listed system
  int* wcoff;               // [nsys + 1] first work item (cell) of each listed system
  int* nwork;               // [3] listed systems, their slots, their cells
  int* status;              // [2] sticky error bits (ST_*), rebuild-chain count
  // the conditional rebuild node of the step a corrector pass belongs to, inside a
  // captured chunk (0 elsewhere): the pass switches it on when a rebuild is due
  unsigned long long cond;
};

// sticky device status bits
enum { ST_NBR_OVERFLOW = 1, ST_NAN = 2, ST_CELL_OVERFLOW = 4, ST_BARRIER_TIMEOUT = 8 };
// spins (of about 64 ns each) a block waits at a grid barrier of the persistent
// step kernel before it gives up, records ST_BARRIER_TIMEOUT and goes on
constexpr unsigned kBarrierSpins = 1u << 24;

constexpr int kScanChunk = 1024;  // cells per scan chunk
constexpr int kSeChunk = 1024;    // particles per reduction chunk
// a system's particle-reduction chunks: [pch0, pch0 + pchunk_count), in slot order
SC_HDI int pchunk_count(const SysGeom& g) { return (g.n + kSeChunk - 1) / kSeChunk; }
constexpr int kMaxCellSort = 48;  // cells above this occupancy use the in-place slow sort
constexpr int kNoTrigger = 0x7f7f7f7f;  // istar value when no particle triggered
constexpr int kOrderWindow = 128;  // slots per window of the force-pass ordering
// mixed-form list entries: slot in the low 28 bits, cell offset (dc+1, dr+1) above
constexpr int kSlotBits = 28;
constexpr unsigned kSlotMask = (1u << kSlotBits) - 1u;
// tile force pass: entry capacity per particle of a tile (compute and read lists
// each), particles and pair results held in shared memory, threads per tile; a
// tile's partner index below kTileInt (bit 27) is a slot, so slots stay below 2^27
constexpr int kTileEPP = 16;
constexpr int kTileCap = 512;
constexpr int kTilePairCap = 2048;
constexpr int kTileThreads = 256;
constexpr unsigned kTileInt = 1u << 27;
constexpr unsigned kTilePayload = kTileInt - 1u;
constexpr unsigned kTileNoEntry = 0xffffffffu;  // a read entry whose pair nobody computes

// pass modes for the force kernels
enum PassMode {
  PASS_FORCE = 0,        // forces at the state positions
  PASS_CORR_STRAIN = 1,  // forces at the predictor copy + Heun corrector (shear)
  PASS_PRED_STRAIN = 2,  // forces at the state + predictor for the next step (shear)
  PASS_CORR_RESIZE = 3,  // forces at the predictor copy + corrector (affine resize,
                         // or pure shear when the row's mode is 3)
  PASS_PRED_RESIZE = 4,  // forces at the state + predictor (affine resize or pure shear)
  PASS_ENERGY_T = 5      // energy (stress partials) at the predictor copy, nothing stored
                         // else (line-search probes of the conjugate-gradient minimiser)
};

// ---- kernel launchers (defined in the .cu files) ----
// tab: device table, row `row` holds nsys StepScalars.
// fast: the minimiser's force evaluation (FORCE mode only), with fewer FP64 divisions
void launch_pass_fp64(const Dev& d, int mode, bool se, const StepScalars* tab, int row,
                      cudaStream_t st, bool fast = false);
void launch_pass_mixed(const Dev& d, int mode, bool se, const StepScalars* tab, int row,
                       cudaStream_t st, int block);
// set-back of the listed systems whose row says so (after launch_rb_worklist)
void launch_setback(const Dev& d, const StepScalars* tab, int row, cudaStream_t st);
// the rebuild worklist: flagged systems and those whose row (tab, row) sets gamma back
void launch_rb_worklist(const Dev& d, const StepScalars* tab, int row, cudaStream_t st);
// the rebuild chain of the listed systems; `listed`: launch_rb_worklist already ran
void launch_rebuild(const Dev& d, bool mixed, const StepScalars* tab, int row, cudaStream_t st,
                    bool listed = false);
void launch_force_rebuild_all(const Dev& d, cudaStream_t st);
void launch_clear_flags(const Dev& d, cudaStream_t st);
void launch_pre_rebuild(const Dev& d, const StepScalars* tab, int row,
                        cudaGraphConditionalHandle cond, cudaStream_t st);
void launch_se_reduce(const Dev& d, cudaStream_t st);
void launch_gd_update(const Dev& d, bool mixed, const StepScalars* tab, int row, cudaStream_t st);
void launch_se_store(const Dev& d, double* dst, cudaStream_t st);
// per-slot values back to input order: out[k * ntot + input index] (k = 0, 1, 2)
void launch_unsort_state(const Dev& d, double* out, cudaStream_t st);
void launch_cg_reset(const Dev& d, const CgState& c, cudaStream_t st);
void launch_cg_begin(const Dev& d, const CgState& c, int max_iter, unsigned long long search,
                     cudaStream_t st);
void launch_cg_probe(const Dev& d, const CgState& c, cudaStream_t st);
void launch_cg_search(const Dev& d, const CgState& c, unsigned long long search,
                      cudaStream_t st);
void launch_cg_move(const Dev& d, const CgState& c, cudaStream_t st);
void launch_ingest(const Dev& d, const double* x, const double* y, const double* phi,
                   const double* R, const double* A, const int* sys_p0, const double* sys_L,
                   int* psys, cudaStream_t st);
void launch_unsort_forces(const Dev& d, double* out, cudaStream_t st);
void launch_refresh_geometry(const Dev& d, bool mixed, const StepScalars* tab, int row,
                             cudaStream_t st);
void launch_build_nbrs(const Dev& d, const StepScalars* tab, int row, cudaStream_t st);
// FIRE and affine rescale
void launch_fire_reset(const Dev& d, const FireState& f, double dt0, cudaStream_t st);
void launch_fire_iteration_tail(const Dev& d, const FireState& f, double ftol, double dt_max,
                                bool mixed, cudaStream_t st);
// factor: 2 nsys entries, the x and y factors of each system
void launch_affine(const Dev& d, const double* factor, cudaStream_t st);
void launch_reflect(const Dev& d, const double* lx, cudaStream_t st);
void launch_rotate(const Dev& d, const double* q, cudaStream_t st);
// mixed form
// all: every slot; else the slots of the listed systems (after launch_rb_worklist)
void launch_mx_materialize(const Dev& d, const StepScalars* tab, int row, bool all,
                           cudaStream_t st);
void launch_mx_local(const Dev& d, const StepScalars* tab, int row, bool all, cudaStream_t st);
void launch_mx_order(const Dev& d, bool all, cudaStream_t st);
// the list build and the ordering in one kernel (the per-particle pass)
void launch_mx_build_order(const Dev& d, const StepScalars* tab, int row, bool all,
                           cudaStream_t st);
void launch_mx_build_list(const Dev& d, const StepScalars* tab, int row, bool all,
                          cudaStream_t st);
// Persistent mixed shear steps (per-particle pass): rows row0 .. row0 + nsteps - 1 of
// the table in one cooperative launch, corrector and predictor passes separated by
// grid barriers, until a step's corrector asks for a rebuild (or a set-back).
// *out = 2 m + stopped: m steps completed, stopped = the corrector of step m + 1 ran
// and its rebuild is pending.  Returns false when the cooperative launch failed.
bool launch_persist_steps(const Dev& d, const StepScalars* tab, int row0, int nsteps, int* out,
                          cudaStream_t st);
// Mixed form: up to `iters` FIRE iterations (force pass, reductions, updates) in one
// cooperative launch of 256-thread blocks, ending early at a pending rebuild or when
// every system has converged.  *out = 4 k + (0 all ran, 1 rebuild pending, 2 all
// converged).  Returns false when the cooperative launch failed.
bool launch_persist_fire(const Dev& d, const FireState& f, const StepScalars* tab, double ftol,
                         double dt_max, int iters, int* out, cudaStream_t st);
// tile lists from the mixed lists (after launch_mx_build_list)
void launch_tile_lists(const Dev& d, bool all, cudaStream_t st);
// FP64 stress and energy partials of the mixed state (two kernels)
void launch_mx_se64(const Dev& d, const StepScalars* tab, int row, cudaStream_t st);

constexpr int kWalkBlocks = 152 * 8;  // fixed grid of the worklist kernels

#ifdef __CUDACC__
// Grid-stride walks over the slots / cells of the systems on the rebuild worklist
// (k_rb_worklist), so that a rebuild of a few systems of a large batch costs in
// proportion to those systems.  f(slot or cell, system).
// the listed system that work item g belongs to (off: exclusive prefix sums)
__device__ __forceinline__ int listed_system(const int* __restrict__ off, int nw, int g) {
  int lo = 0, hi = nw - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}
template <class F>
__device__ __forceinline__ void for_listed_slots(const Dev& d, F&& f) {
  const int nw = d.nwork[0], W = d.nwork[1];
  const int t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int g = t; g < W; g += stride) {
    const int w = listed_system(d.woff, nw, g);
    const int s = d.work[w];
    f(d.geom[s].p0 + (g - d.woff[w]), s);
  }
}
template <class F>
__device__ __forceinline__ void for_listed_cells(const Dev& d, F&& f) {
  const int nw = d.nwork[0], W = d.nwork[2];
  const int t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int g = t; g < W; g += stride) {
    const int w = listed_system(d.wcoff, nw, g);
    const int s = d.work[w];
    f(d.geom[s].c0 + (g - d.wcoff[w]), s);
  }
}
// Corrector passes inside a captured step (d.cond != 0), block 0 before any early
// exit: mark the systems that set gamma back at this step (their rows say so) and
// switch the step's rebuild node on for them, or for a rebuild still pending.
__device__ __forceinline__ void mark_pending_rebuilds(const Dev& d,
                                                      const StepScalars* __restrict__ tab,
                                                      int row) {
  if (!d.cond || blockIdx.x != 0) return;
  bool setback = false;
  for (int s = threadIdx.x; s < d.nsys; s += blockDim.x)
    if (tab[row * d.nsys + s].setback) {
      atomicOr(&d.flags[s], 2);
      setback = true;
    }
  if (setback) atomicExch(d.any, 1);
  if (setback || (threadIdx.x == 0 && *d.any != 0)) cudaGraphSetConditional(d.cond, 1u);
}
// A particle of system s needs its list rebuilt: flag the system, raise the pending
// word, and (the thread that raises it) switch the step's rebuild node on.
__device__ __forceinline__ void request_rebuild(const Dev& d, int s) {
  if (d.flags[s] == 0) atomicOr(&d.flags[s], 1);
  if (*d.any == 0 && atomicExch(d.any, 1) == 0 && d.cond) cudaGraphSetConditional(d.cond, 1u);
}
// all: every slot of every system (forced refreshes), else the worklist
template <class F>
__device__ __forceinline__ void for_slots(const Dev& d, bool all, F&& f) {
  if (!all) {
    for_listed_slots(d, f);
    return;
  }
  const int t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int i = t; i < d.ntot; i += stride) f(i, d.psys[i]);
}
#endif

}  // namespace sc
