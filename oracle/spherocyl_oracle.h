/*
 * spherocyl_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * C interface of the CPU restatement of tmarschall/spherocyls' src/cpp path
 * (spherocyl_oracle.c).  Only tests, the smoke check and the CPU-baseline leg of
 * the benchmark use it, as the oracle; the product library never links it.
 */
#ifndef SPHEROCYL_ORACLE_H
#define SPHEROCYL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_box orc_box;

orc_box *orc_create(int n, double L, const double *x, const double *y, const double *phi,
                    const double *A, const double *R, double pad);
orc_box *orc_create_rect(int n, double Lx, double Ly, const double *x, const double *y,
                         const double *phi, const double *A, const double *R, double pad);
void orc_destroy(orc_box *b);

void orc_set_strain_rate(orc_box *b, double v);
void orc_set_resize_rate(orc_box *b, double v);
void orc_set_step(orc_box *b, double v);
void orc_set_gamma(orc_box *b, double v);
void orc_set_total_gamma(orc_box *b, double v);
void orc_zero_pyx(orc_box *b);
void orc_set_two_point(orc_box *b, int on);

void orc_find_neighbors(orc_box *b);
void orc_calc_forces(orc_box *b);
void orc_calc_se(orc_box *b);
int orc_strain_step(orc_box *b);
long orc_strain_to_gamma(orc_box *b, double gamma_max);
int orc_resize_step(orc_box *b, int shrink);
int orc_gd_step(orc_box *b);
int orc_pure_step(orc_box *b);

int orc_run_strain_steps(orc_box *b, int nsteps, double *se_out);
int orc_run_resize_steps(orc_box *b, int nsteps, int shrink, double *se_out);
int orc_run_gd_steps(orc_box *b, int nsteps, double emin, double *e_out);
int orc_run_pure_steps(orc_box *b, int nsteps, double *se_out);
int orc_cg_minimize(orc_box *b, int max_iter, int *iters, double *e_out, int *reason);

int orc_n(const orc_box *b);
void orc_get_state(const orc_box *b, double *x, double *y, double *phi);
void orc_get_forces(const orc_box *b, double *fx, double *fy, double *tau);
void orc_get_moved(const orc_box *b, double *xm, double *ym);
void orc_get_consts(const orc_box *b, double *I, double *RC);
void orc_get_scalars(const orc_box *b, double *out);
void orc_get_se(const orc_box *b, double *out);
long orc_get_pairs(const orc_box *b, int *pairs, long cap);
long orc_n_rebuilds(const orc_box *b);

/* The benchmark workload's input packing (seeded, crossing-free; the same packing as
 * the library's sc_generate_packing).  Returns 0 on success. */
int orc_generate_packing(int n, double packing, double a_over_r, double r_small, double r_ratio,
                         uint64_t seed, double min_sep, double *x, double *y, double *phi,
                         double *R, double *A, double *L_out);

#ifdef __cplusplus
}
#endif

#endif
