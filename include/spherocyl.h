/*
 * spherocyl.h -- C ABI of libspherocyl, the GB300 (sm_103a) implementation of the
 * overdamped-dynamics hot path of tmarschall/spherocyls: 2D bidisperse
 * spherocylinder packings under Lees-Edwards simple shear and affine box resize,
 * plus energy minimisation.
 *
 * The reference has no library API; its callers are the CLI drivers, which build
 * one box object and call one run method (src/cpp/main.cpp:63-196,
 * src/cpp/main_resize.cpp:63-193, src/cpp/main_relax.cpp:63-181).  Each entry
 * point below names the reference routine it replaces.  One handle holds one or
 * more independent periodic boxes ("systems") that advance together; with one
 * system a handle is a drop-in for SpherocylBox (src/cpp/spherocyl_box.h:26-122).
 *
 * Conventions
 *  - Every function returns an int status (SC_OK == 0) and never exits or aborts;
 *    sc_last_error() gives a one-line description of the last failure.
 *  - Arrays are plain host pointers, copied on entry; the library owns all device
 *    memory and never keeps a caller pointer.
 *  - Per-particle arrays concatenate the systems in order, each in the reference's
 *    particle order.  "sys" arguments take a system index or -1 for all systems.
 *  - A handle is used by one host thread at a time; its work runs on its own CUDA
 *    stream (or the stream given to sc_set_stream).
 */
#ifndef SPHEROCYL_H
#define SPHEROCYL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference's exit(1)/assert/checkCudaError paths,
 *      src/cuda/cudaErr.cpp:11-19, become these) ---- */
#define SC_OK 0
#define SC_E_ARG 1      /* invalid argument */
#define SC_E_IO 2       /* file could not be read or written */
#define SC_E_NAN 3      /* a position or angle became non-finite */
#define SC_E_OVERFLOW 4 /* neighbour list or cell capacity exceeded */
#define SC_E_NOCONV 5   /* minimiser stopped at its iteration cap, or a jamming
                           bisection's step grew to 1 without crossing its target */
#define SC_E_TIMEOUT 6  /* a bounded device wait gave up */
#define SC_E_CUDA 7     /* CUDA runtime error */
#define SC_E_STATE 8    /* call not valid in the handle's current state */
#define SC_E_NOMEM 9    /* host or device allocation failed */

#define SC_PREC_FP64 0  /* plain FP64: the reference's arithmetic, step for step */
#define SC_PREC_MIXED 1 /* FP32 pair geometry, FP64 state and accumulators */

#define SC_STRESS_COMPAT 0 /* stress exactly as src/cpp accumulates it (with its slips) */
#define SC_STRESS_VIRIAL 1 /* the intended contact virial */

#define SC_CONTACT_ONE 0 /* one closest-point contact per pair (src/cpp) */
#define SC_CONTACT_TWO 1 /* up to two contacts per pair for near-parallel spines
                          * (src/cuda/2point_dynamics.cu:385-546), used for jamming */

#define SC_FMT_SP 0 /* src/cpp position file: "N L phi gamma gamma_tot rate dt" */
#define SC_FMT_SD 1 /* src/cuda position file: "N Lx Ly phi gamma gamma_tot rate dt" */
#define SC_FMT_BIN 2 /* src/cuda binary position file (save_positions_bin,
                      * src/cuda/strain_dynamics.cu:845-875): int N, then the sd header's
                      * seven doubles, then x y phi R A as doubles per particle */

typedef struct sc_handle sc_handle;

typedef struct sc_options {
  int precision;   /* SC_PREC_* */
  int stress_mode; /* SC_STRESS_* */
  int device;      /* CUDA device ordinal */
  int max_nbrs;    /* FP64 neighbour-list capacity per particle, 0 = default (64) */
  int use_graphs;  /* capture step chunks in CUDA graphs (1) or launch eagerly (0) */
  int block;       /* threads per block of the mixed force pass (<= 128), 0 = 128 */
  int profile;     /* record per-pass CUDA events inside run calls (sc_get_pass_times) */
  int contact_model; /* SC_CONTACT_* */
  int stage_inputs;  /* 1: copy the input arrays to the device before building the state,
                      * also where the GPU reads pageable host memory in place (0) */
  int cg_max_probes; /* energy probes one conjugate-gradient line search may take before
                      * its system stops with SC_CG_PROBES, 0 = default (256) */
  int pass_kind;     /* mixed form's force pass: SC_PASS_LIST (one thread per particle
                      * over its full list, each pair twice), SC_PASS_TILE (blocks of
                      * cells staged in shared memory, each pair inside a tile once) or
                      * SC_PASS_AUTO (the list pass until sc_autotune times both) */
  int tile_target;   /* particles per tile the tile pass aims at, 0 = default (256) */
  int persist_steps; /* mixed form, per-particle pass, simple shear: 1 advances runs of
                      * steps in one persistent cooperative launch (corrector and
                      * predictor passes separated by bounded grid barriers) until a
                      * step needs a rebuild; 0 launches each pass (CUDA graphs) */
} sc_options;

#define SC_PASS_AUTO 0
#define SC_PASS_LIST 1
#define SC_PASS_TILE 2

const char *sc_version(void);
const char *sc_status_string(int status);
void sc_default_options(sc_options *opt);

/* Create a handle holding n_sys periodic square boxes of side L[s] and padding
 * pad[s] (0 = automatic, as configure_cells, src/cpp/spherocyl_box.cpp:240-241).
 * Replaces SpherocylBox(L, N, x, y, phi, A*, R*, pad), src/cpp/spherocyl_box.cpp:152-173:
 * positions and angles are wrapped, MOI and rotation coefficients derived
 * (set_particle :188-221), cells configured (:223-268) and lists built (:320-355). */
int sc_create(const sc_options *opt, int n_sys, const int *n_per_sys, const double *L,
              const double *pad, const double *x, const double *y, const double *phi,
              const double *R, const double *A, sc_handle **out);
/* As sc_create for rectangular boxes Lx[s] x Ly[s] (the src/cuda box,
 * src/cuda/spherocyl_box.cpp:529-636): the Lees-Edwards set-back then happens at
 * gamma >= Lx/(2 Ly) and subtracts Lx/Ly (set_back_coords, src/cuda/find_neighbors.cu:285-330);
 * for Lx = Ly it is sc_create. */
int sc_create_rect(const sc_options *opt, int n_sys, const int *n_per_sys, const double *Lx,
                   const double *Ly, const double *pad, const double *x, const double *y,
                   const double *phi, const double *R, const double *A, sc_handle **out);
int sc_destroy(sc_handle *h);
/* Device memory of all handles on a device comes from one stream-ordered pool that
 * keeps the blocks of destroyed handles for the next one (creating a handle of a
 * size seen before then allocates nothing).  sc_trim_memory returns the unused
 * blocks to the driver. */
int sc_trim_memory(int device);
const char *sc_last_error(const sc_handle *h);
int sc_set_stream(sc_handle *h, void *cuda_stream);
int sc_synchronize(sc_handle *h);

/* Setters, src/cpp/spherocyl_box.h:112-119 (set_strain_rate, set_resize_rate,
 * set_step, set_cell_padding, set_gamma, set_total_gamma). */
int sc_set_strain_rate(sc_handle *h, int sys, double v);
int sc_set_resize_rate(sc_handle *h, int sys, double v);
int sc_set_step(sc_handle *h, int sys, double v);
int sc_set_gamma(sc_handle *h, int sys, double v);
int sc_set_total_gamma(sc_handle *h, int sys, double v);

/* find_neighbors, src/cpp/spherocyl_box.cpp:320-355 (forced rebuild). */
int sc_find_neighbors(sc_handle *h);
/* calc_forces, src/cpp/strain_dynamics.cpp:137-153. */
int sc_calc_forces(sc_handle *h);
/* calc_se, src/cpp/spherocyl_box.cpp:502-522: forces plus per-system
 * E, Pxx, Pyy, Pxy, Pyx written to se_out[5*s + k] (se_out may be NULL). */
int sc_calc_se(sc_handle *h, double *se_out);

/* nsteps Heun steps under Lees-Edwards shear: strain_step followed by
 * calc_forces, or calc_se every se_every steps (run_strain's inner loop,
 * src/cpp/strain_dynamics.cpp:179-235 and :285-296).  When se_every > 0 and
 * se_out != NULL, se_out receives (nsteps/se_every) records of 5*n_sys values. */
int sc_strain_steps(sc_handle *h, int nsteps, int se_every, double *se_out);
/* Shear without setting gamma back until gamma >= gamma_max (run_strain(dGammaMax),
 * src/cuda/strain_dynamics.cu:1097-1108, the strain driver's shear-direction change
 * 3 before rotate_by_gamma), on cells 2 sqrt(1 + gamma_max^2)(R_max + A_max) + pad
 * wide, which the handle keeps.  One system per handle; *steps receives the steps
 * taken. */
int sc_strain_to_gamma(sc_handle *h, double gamma_max, long *steps);
/* nsteps Heun steps with affine resize by (1-rate)^dt per step (shrink != 0) or its
 * inverse (resize_step + calc_forces, src/cpp/resize_dynamics.cpp:164-243, :297-307). */
int sc_resize_steps(sc_handle *h, int nsteps, int shrink, int se_every, double *se_out);
/* nsteps pure-shear steps at each system's strain rate e (pure_strain_step_2p,
 * src/cuda/2point_dynamics.cu:1664-2283): the predictor adds the flow (+e x/2,
 * -e y/2) and the isolated rotation -e RC sin(2 phi)/2 to the contact motion, the
 * corrector adds dt/2 times the change of the contact forces evaluated in the
 * predicted box Lx(1 + dt e/2) x Ly(1 - dt e/2); then Lx += dt e Lx/2,
 * Ly -= dt e Ly/2, gamma_total += dt e (gamma is unchanged).  Unit drag and the
 * torque over I, as in the other steps; the contact model is the handle's.
 * Records as sc_strain_steps.  Replaces Spherocyl_Box::pure_strain_step_2p. */
int sc_pure_strain_steps(sc_handle *h, int nsteps, int se_every, double *se_out);
/* Fixed-step gradient descent (gradient_descent_minimize's loop,
 * src/cpp/relaxation_dynamics.cpp:11-85): calc_se, stop when every system's
 * E <= e_min, else x += dt F.  *steps_taken receives the iterations done. */
int sc_gd_minimize(sc_handle *h, int max_steps, double e_min, int *steps_taken,
                   double *e_final);

/* Polak-Ribiere conjugate gradient with the reference's line search
 * (cjpr_relax_2p / cjpr_relax_step_2p / line_search_2p,
 * src/cuda/2point_dynamics.cu:3609-3780, 3886-4020, 4233-4296), FP64 form, every
 * system at once and entirely on the device.  Per iteration: D = F + beta D with
 * beta = max(0, (F.F - F.F0)/F0.F0) (restarted every 3N iterations); a line search
 * from 2e-6/|F|_rms, doubling while the energy falls and halving while it rises
 * (within [1e-18, 2]/|F|_rms), then the minimum of the parabola through E(0), E(s),
 * E(2s); on failure steepest descent, then F/sqrt|F|.  A system stops at zero force
 * (reason SC_CG_ZERO_FORCE), three equal iteration energies (SC_CG_STALLED), no
 * lower energy in any direction (SC_CG_STEP) or max_iter iterations
 * (SC_CG_MAX_ITER).  A line search that still asks for another energy probe after
 * sc_options.cg_max_probes probes (the reference's search has no such cap; its step
 * limits end it within about 135) stops its system with SC_CG_PROBES.  iters, energy
 * (the calc_se energy at the end) and reason take n_sys entries each and may be NULL.
 * Returns SC_E_NOCONV when a system reached max_iter or the probe cap. */
#define SC_CG_ZERO_FORCE 1
#define SC_CG_STALLED 2
#define SC_CG_STEP 3
#define SC_CG_MAX_ITER 4
#define SC_CG_PROBES 5
int sc_cg_minimize(sc_handle *h, int max_iter, int *iters, double *energy, int *reason);
/* Production minimiser: FIRE on every system of the handle, on the device, until
 * every |F_i| and |tau_i|/sqrt(I_i) is below ftol, or max_iter iterations.  Replaces
 * the reference's conjugate-gradient relaxation (cjpr_relax_2p,
 * src/cuda/2point_dynamics.cu:4233-4295), whose line search returns to the host on
 * every probe.  dt0/dt_max: initial and largest FIRE step.  Per-system outputs
 * (may be NULL): fmax[s], done[s]; *iters the most iterations any system took.
 * Returns SC_E_NOCONV when some system did not reach ftol. */
int sc_fire_minimize(sc_handle *h, double ftol, int max_iter, double dt0, double dt_max,
                     int *iters, double *fmax, int *done);
/* Iterations each system took in the handle's last sc_fire_minimize (up to and
 * including the one that brought it below ftol): iters[s], s < the system count.
 * All zero before the first call. */
int sc_fire_iterations(const sc_handle *h, int *iters);
/* Affine rescale of box and positions by factor (the src/cuda resize_coords,
 * src/cuda/strain_dynamics.cu:1111-1122, as one step); sys = -1 for all. */
int sc_affine_scale(sc_handle *h, int sys, double factor);
/* flip_shear_direction (src/cuda/find_neighbors.cu:563-581): reverses the shear of
 * system sys (-1: all) by reflecting x -> Lx - x, phi -> -phi and gamma -> -gamma;
 * the cell lists are rebuilt.  Shear then continues with the same strain rate. */
int sc_flip_shear(sc_handle *h, int sys);
/* rotate_by_gamma (src/cuda/find_neighbors.cu:583-645): turns system sys (-1: all)
 * to the frame in which its sheared cell is upright, Lx' = Ly sqrt(1 + gamma^2),
 * Ly' = Lx / sqrt(1 + gamma^2), gamma -> -gamma (the box becomes rectangular). */
int sc_rotate_shear(sc_handle *h, int sys);
/* Quasistatic compression to jamming: repeated affine steps raising each system's
 * packing fraction by dphi, each followed by sc_fire_minimize(ftol, max_iter), until
 * the system's energy per particle exceeds e_jam (compress_qs2p / find_jam_2p,
 * src/cuda/2point_dynamics.cu:4299-4344, 4582-4606).  phi_jam[s] receives the
 * packing fraction at which system s jammed (negated when max_increments ran out);
 * *n_inc the increments made. */
int sc_quasistatic_compress(sc_handle *h, double dphi, double ftol, double e_jam,
                            int max_increments, int max_iter, double *phi_jam, int *n_inc);
/* find_jam_2p / resize_to_energy_2p (src/cuda/2point_dynamics.cu:4582-4606,
 * 4393-4456): per system, affine length factors 1 - step to compress and
 * 1/(1 - step) to expand (resize_step_2p), the step growing by 1.1 per resize and
 * FIRE to ftol after each, towards energy per particle e_jam, reversing with
 * half the last step each time the energy crosses e_jam, until the step is below
 * min_step or max_steps resizes were made.  phi_jam[s]: final packing fraction of
 * system s (negated when max_steps ran out first); *steps: resizes made.
 * SC_E_NOCONV if a step grows to 1 before the energy crosses e_jam. */
int sc_find_jam(sc_handle *h, double e_jam, double step, double min_step, double ftol,
                int max_iter, int max_steps, double *phi_jam, int *steps);

/* Mixed form: times `steps` shear steps (after as many warm-up steps) of a copy of
 * the handle for each candidate -- padding factors {0.5, 1, 1.5, 2, 3} x the current
 * padding, crossed with the per-particle force pass at block sizes {64, 128}, the
 * same pass in the persistent step kernel, and the tile force pass at {128, 256, 384}
 * particles per tile -- and gives the handle the fastest (*pad_factor, *block; the
 * pass kind, tile size and persistence through sc_get_options).  The live state is not advanced.  The FP64 form is left as it is
 * (factor 1).  Replaces the reference's fixed launch-shape table
 * (src/cuda/spherocyl_box.cpp:193-238). */
int sc_autotune(sc_handle *h, int steps, double *pad_factor, int *block);
/* The handle's current options (after sc_autotune: the chosen pass kind, block and
 * tile size). */
int sc_get_options(const sc_handle *h, sc_options *out);

/* State readers, original particle order, systems concatenated. */
int sc_get_state(sc_handle *h, double *x, double *y, double *phi);
int sc_get_forces(sc_handle *h, double *fx, double *fy, double *tau);
/* Per-system scalars: out[0..9] = Lx Ly gamma gamma_total pad W H packing rows cols. */
int sc_get_box(sc_handle *h, int sys, double *out);
/* Half neighbour list of one system as (p, q) pairs with p < q, sorted; with
 * pairs == NULL only *n_pairs is written.  (The reference's m_pvNeighbors.) */
int sc_get_pairs(sc_handle *h, int sys, int *pairs, long cap, long *n_pairs);
/* Counters: out[0] steps, out[1] rebuild chains executed on the device, out[2]
 * device status bits, out[3] kernels launched so far. */
int sc_get_counters(sc_handle *h, long long *out);
/* Mean device time per force pass of the last run call with profiling on:
 * out[0] corrector passes (ms), out[1] predictor passes (ms), out[2] rebuild
 * chains (ms), out[3..5] the number of each. */
int sc_get_pass_times(sc_handle *h, double *out);

/* Seeded crossing-free random packing: species alternate by index (R = r_small
 * for even, r_small*r_ratio for odd indices), A = a_over_r * R, L from the packing
 * fraction sum(pi R^2 + 4 A R)/L^2, centres uniform, angles uniform in [0, pi),
 * a placement rejected while its spine comes closer than min_sep * (R_i + R_j) to
 * an earlier spine.  Replaces random_configuration's rand()/time(0) placement
 * (src/cpp/spherocyl_box.cpp:694-790) with a reproducible one. */
int sc_generate_packing(int n, double packing, double a_over_r, double r_small, double r_ratio,
                        uint64_t seed, double min_sep, double *x, double *y, double *phi,
                        double *R, double *A, double *L);

/* The reference's initial configurations (place_spherocyls, place_random_0e_spherocyls,
 * place_spherocyl_grid, set_shapes, uniformToAngleDist:
 * src/cuda/spherocyl_box.cpp:1044-1394), seeded and reproducible. */
#define SC_LAYOUT_RANDOM 0 /* centres uniform in the box */
#define SC_LAYOUT_GRID 1   /* one particle per grid cell, rows offset at random */
#define SC_ANGLE_RANDOM 0  /* u uniform in [angle_min, angle_max] */
#define SC_ANGLE_EVEN 1    /* u = angle_min + (2i+1)(angle_max - angle_min)/(2n) */
/* sc_generate_packing's packing (same shapes, box and rejection rule) placed on GPU
 * `device` in rounds: every particle still to place draws from a counter-based hash
 * of (seed, particle, round), and is redrawn while its spine comes closer than
 * min_sep (R_i + R_j) to that of a lower-numbered particle (for large N; the host
 * placement is sequential).  Deterministic for a seed, but not the host's sequence.
 * min_sep = 1 gives zero-energy (contact-free) placement.  SC_E_ARG for a box of
 * fewer than 3 reach-wide cells, SC_E_NOCONV past the placement's saturation. */
int sc_generate_packing_device(int device, int n, double packing, double a_over_r,
                               double r_small, double r_ratio, uint64_t seed, double min_sep,
                               double *x, double *y, double *phi, double *R, double *A,
                               double *L);

typedef struct sc_gen_options {
  int layout;         /* SC_LAYOUT_* */
  int angle_mode;     /* SC_ANGLE_*; angle_min == angle_max gives aligned particles */
  double angle_min;   /* u range in [0, 1]; the angle is pi u - pi/2, or with     */
  double angle_max;   /* shear_angles the isolated-rotation steady-shear quantile */
  int shear_angles;
  double min_sep;     /* reject spine distances below min_sep (R_i + R_j) */
  double max_overlap; /* >= 0: also reject d^2 < (1 - max_overlap)(R_i + R_j)^2
                       * (0 = zero energy); < 0: off */
  double a_sigma;     /* > 0: a/R Gamma-distributed, mean a_over_r, std a_sigma*a_over_r */
} sc_gen_options;
void sc_default_gen_options(sc_gen_options *opt); /* random, u in [0,1], min_sep 0.1 */
int sc_generate_config(const sc_gen_options *opt, int n, double packing, double a_over_r,
                       double r_small, double r_ratio, uint64_t seed, double *x, double *y,
                       double *phi, double *R, double *A, double *L);
/* The same in a rectangle of aspect box_aspect = Lx/Ly and area L^2 (the
 * pure-shear driver starts at Lx/Ly = 1/stop_aspect, src/cuda/main_pure_shear.cpp:
 * 168-170); box_aspect = 1 gives sc_generate_config's packing. */
int sc_generate_config_rect(const sc_gen_options *opt, int n, double packing, double a_over_r,
                            double r_small, double r_ratio, double box_aspect, uint64_t seed,
                            double *x, double *y, double *phi, double *R, double *A, double *Lx,
                            double *Ly);

/* ---- files and run protocols with output (single-system handles) ---- */

/* Read a position file (DatFileInput with a header row, src/cpp/file_input.h:24-76).
 * Both header layouts are accepted: the src/cpp one, "N L packing gamma
 * gamma_total rate dt" (7 fields), and the src/cuda one, "N Lx Ly packing gamma
 * gamma_total rate dt" (8 fields, src/cuda/main.cpp:201).  Rows are "x y phi R A".
 * Call once with x == NULL to get *n and hdr; then with arrays of *n entries.
 * hdr[0..6] = Lx Ly packing gamma gamma_total rate dt. */
int sc_read_positions(const char *path, int *n, double *hdr, double *x, double *y, double *phi,
                      double *R, double *A);
/* save_positions: SC_FMT_SP as src/cpp/spherocyl_box.cpp:410-423 (precision 14; a
 * rectangular box gets the src/cuda header's Lx and Ly),
 * SC_FMT_SD as src/cuda/strain_dynamics.cu:820-843 (%.17g rows), SC_FMT_BIN as
 * src/cuda/strain_dynamics.cu:845-875 (host byte order).  sc_read_positions reads a
 * path ending in ".bin" as SC_FMT_BIN, one ending in ".gz" as gzip-compressed text
 * (GzFileInput, src/cpp/gz_file_input.cpp; needs libz.so.1 at run time), any other
 * as text with either header. */
int sc_save_positions(sc_handle *h, int sys, const char *path, int format);
/* The same files from host arrays, without a handle (a configuration made on the
 * host, src/cuda/main_configmaker.cpp's use): hdr[0..6] = Lx Ly packing gamma gamma_total
 * rate dt as sc_read_positions gives them, n rows "x y phi R A".  Errors: SC_E_ARG,
 * SC_E_IO, with sc_last_error(NULL) text. */
int sc_write_positions(const char *path, int format, int n, const double *hdr, const double *x,
                       const double *y, const double *phi, const double *R, const double *A);

/* run_strain with output, src/cpp/strain_dynamics.cpp:238-319: t runs from t_start
 * to t_start + round(run_gamma/rate) in units of 1/dt steps; stress/energy lines
 * every se_save strain (SE file sp_strain_se.dat, or sd_stress_energy.dat for
 * SC_FMT_SD) and position files every pos_save strain, named sp%010lu.dat /
 * sd%010lu.dat; t_start > 0 continues an earlier run, rewriting the SE file from
 * the line of time t_start.  *t_end receives the final time. */
int sc_run_strain(sc_handle *h, const char *out_dir, double run_gamma, double pos_save,
                  double se_save, unsigned long t_start, int format, unsigned long *t_end);
/* resize_box with output, src/cpp/resize_dynamics.cpp:246-330 (SE file
 * sp_resize_se.dat with the packing fraction as second column). */
int sc_run_resize(sc_handle *h, const char *out_dir, double final_packing, double pos_save,
                  double se_save, unsigned long t_start, int format, unsigned long *t_end);
/* run_pure_strain_2p with output, src/cuda/2point_dynamics.cu:2286-2391: pure
 * shear until Lx/Ly >= stop_aspect, in time units of 1/dt steps; SE lines (format
 * and file as sc_run_strain) for the states after every multiple of se_save/(e dt)
 * steps and at each position save; position files every pos_save/e time units and
 * of the final state.  t_start > 0 continues as sc_run_strain.  A negative rate is
 * used as its magnitude.  *t_end receives the final time. */
int sc_run_pure_strain(sc_handle *h, const char *out_dir, double stop_aspect, double pos_save,
                       double se_save, unsigned long t_start, int format, unsigned long *t_end);
/* find_jam_2p with output, src/cuda/2point_dynamics.cu:4393-4456, 4582-4606, for a
 * one-system handle: the bisection of sc_find_jam (min_step 1e-15) towards e_jam
 * given, as there, as calc_fe_2p's energy per unit area (E/N x N / 2LxLy); each
 * resize relaxes with sc_cg_minimize(max_iter) in the FP64 form (cjpr_relax_2p) and
 * FIRE to ftol in the mixed form.  Writes sd0000000000.dat, then per resize t a line
 * "t packing E Pxx Pyy Pxy Pyx" (E per unit area) in sd_stress_energy.dat and
 * sd%010d.dat, and the final state as sd%010d.bin.  *steps: resizes made; *phi_jam:
 * final packing fraction (negated if the step limit of 10^6 resizes ran out). */
int sc_run_find_jam(sc_handle *h, const char *out_dir, double e_jam, double step,
                    double ftol, int max_iter, int *steps, double *phi_jam);
/* y_compress_energy_2p with output, src/cuda/2point_dynamics.cu:4458-4530, 4608-4631:
 * sc_run_find_jam's bisection and files with resizes of Ly and the y coordinates
 * alone (y_resize_step_2p: factors 1 - step and 1/(1 - step)), towards the energy
 * per unit area e_target, until the step is below 1e-14.  *packing: the final
 * packing fraction (negated if 10^6 resizes ran out). */
int sc_run_y_compress(sc_handle *h, const char *out_dir, double e_target, double step,
                      double ftol, int max_iter, int *steps, double *packing);
/* compress_qs2p / expand_qs2p with output, src/cuda/2point_dynamics.cu:4296-4391,
 * for a one-system handle: relaxation, then affine resizes by the length factor
 * 1 - |step| (compression, final_packing above the current packing fraction) or
 * 1/(1 - |step|) (expansion), each followed by a relaxation -- sc_cg_minimize(max_iter)
 * in the FP64 form (cjpr_relax_2p), FIRE to ftol in the mixed form -- until the
 * packing fraction reaches final_packing.  The start and each resize t write a line
 * "t packing E Pxx Pyy Pxy Pyx" (E per unit area, as sc_run_find_jam) in
 * sd_stress_energy.dat and sd%010d.dat.  *steps: resizes made. */
int sc_run_qs_compress(sc_handle *h, const char *out_dir, double final_packing, double step,
                       double ftol, int max_iter, int *steps);
/* gradient_descent_minimize with output, src/cpp/relaxation_dynamics.cpp:33-85 (SE
 * file sr_strain_se.dat, position files sr%010lu.dat every pos_save_n steps). */
int sc_run_minimize(sc_handle *h, const char *out_dir, int max_steps, double e_min,
                    int pos_save_n, int *steps_taken);

/* ---- allocation-free force evaluation (no counterpart in the reference) ----
 * For callers that cannot let a library allocate device memory -- a host program
 * that has divided the GPU's memory among its own solvers and passes only
 * pre-allocated buffers, or a loop that must never reach the allocator.  Computes,
 * for one periodic square box of side L at shear offset gamma, the contact forces
 * and torques that sc_calc_forces gives on an FP64 handle, from caller-owned device
 * arrays (x, y, phi, R, A in; fx, fy, tau out; n entries each) on the given stream
 * (NULL: the default stream), asynchronously.  The cell lists live in one fixed
 * file-scope device array (about 0.9 MB, resident on every GPU that loads the
 * library until the process exits); no cudaMalloc, cudaFree or other allocation is
 * made.  n above SC_NOALLOC_MAX_PARTICLES is rejected with SC_E_ARG, and so is a
 * non-finite gamma.  Any gamma is served: past |gamma| = 1/2 the cells widen to
 * 2 sqrt(1 + gamma^2)(R_max + A_max) + pad, the width the handle's grid takes for
 * shear past 1/2 (sc_strain_to_gamma).  A box only a few cells wide (large R + A
 * against L) sorts each crowded cell on one thread, so such calls are slow for
 * large n.  The first call on a device looks up the array's address on that device
 * and keeps it for the process: make that call before any stream capture, and make
 * no call on a device after cudaDeviceReset on it.  Calls share the array, so calls
 * that overlap on the GPU race; serialise them.  sc_noalloc_last_error() describes
 * the last failure. */
#define SC_NOALLOC_MAX_PARTICLES 65536
int sc_forces_noalloc(int n, double L, double gamma, double pad, const double *d_x,
                      const double *d_y, const double *d_phi, const double *d_R,
                      const double *d_A, double *d_fx, double *d_fy, double *d_tau,
                      void *cuda_stream);
const char *sc_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SPHEROCYL_H */
