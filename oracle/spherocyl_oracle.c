/*
 * spherocyl_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C restatement of the single-threaded CPU path of tmarschall/spherocyls
 * (src/cpp).  The tests, the smoke check and the CPU-baseline leg of the benchmark
 * use it as the oracle the CUDA library is compared with.  It is never linked into, or called
 * by, the product library.
 *
 * Every routine follows one reference routine and cites it.  Arithmetic is written
 * so that the floating-point operations and their order are the reference's
 * (compiled with -ffp-contract=off), which makes the restatement bit-identical to
 * the compiled reference on the same machine; tests/test_oracle_pin.py checks that
 * against fixtures produced by the reference itself (tests/golden/).
 *
 * State is one box: SoA arrays in the reference's particle order.  The half
 * neighbour list is a growable array per particle, filled in the reference's
 * traversal order (own cell, then the 8 neighbour cells in table order).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "spherocyl_oracle.h"

/* The reference's truncated pi (src/cpp/spherocyl_box.cpp:12).  Its value enters
 * the moment of inertia, the rotation coefficient and the angle wrap, so the
 * oracle uses the same constant to stay bit-identical. */
static const double REF_PI = 3.14159265358979;

typedef struct {
  int *data;
  int len, cap;
} ivec;

static int ivec_push(ivec *v, int x) {
  if (v->len == v->cap) {
    int nc = v->cap ? 2 * v->cap : 8;
    int *nd = (int *)realloc(v->data, (size_t)nc * sizeof(int));
    if (!nd) return -1;
    v->data = nd;
    v->cap = nc;
  }
  v->data[v->len++] = x;
  return 0;
}

static void ivec_free_array(ivec *v, int n) {
  if (!v) return;
  for (int i = 0; i < n; i++) free(v[i].data);
  free(v);
}

struct orc_box {
  int n;
  double Lx, Ly;
  double gamma, gamma_total, strain_rate, resize_rate, step, pad;
  double Rmax, Amax, packing;
  int rows, cols, ncells;
  double W, H;
  /* particles (the reference's Spherocyl struct, src/cpp/spherocyl_box.h:10-24) */
  double *x, *y, *phi, *R, *A, *I, *RC, *fx, *fy, *tau, *xm, *ym;
  int *cell;
  /* the copy used by the Heun predictor (m_psTempParticles) */
  double *tx, *ty, *tphi, *tfx, *tfy, *ttau;
  ivec *cells;     /* per-cell particle lists, ncells of them */
  int *cell_nbrs;  /* 8 neighbour cells per cell */
  ivec *nbrs;      /* per-particle half lists */
  double E, Pxx, Pyy, Pxy, Pyx;
  long n_rebuilds;
  int err;
  int two_point; /* contact model: 0 one point (src/cpp), 1 two points (src/cuda 2p) */
  double wfac;   /* cell width over Rmax + Amax: 2.24 (src/cpp), 2 sqrt(1 + g^2) for a run
                  * to gamma g (src/cuda/spherocyl_box.cpp:132-144) */
  int no_setback; /* shear past gamma = 1/2 (run_strain(dGammaMax)) */
};

/* ---- per-particle constants and wrap: set_particle, spherocyl_box.cpp:188-221 ---- */
static void wrap_particle(orc_box *b, int p) {
  /* the wrap loops of set_particle :204-215, repeated in find_cells :279-290 */
  while (b->x[p] > b->Lx) b->x[p] -= b->Lx;
  while (b->x[p] < 0.0) b->x[p] += b->Lx;
  while (b->y[p] > b->Ly) b->y[p] -= b->Ly;
  while (b->y[p] < 0.0) b->y[p] += b->Ly;
  while (b->phi[p] > REF_PI) b->phi[p] -= 2 * REF_PI;
  while (b->phi[p] < -REF_PI) b->phi[p] += 2 * REF_PI;
}

static void set_particle(orc_box *b, int p, double x, double y, double phi, double A, double R) {
  b->x[p] = x;
  b->y[p] = y;
  b->phi[p] = phi;
  b->A[p] = A;
  b->R[p] = R;
  double al = A / R;
  double C = (3 * REF_PI + 24 * al + 6 * REF_PI * al * al + 8 * al * al * al);
  double area = R * (REF_PI * R + 4 * A);
  b->I[p] = R * R * R * R * C / (6 * area);
  b->RC[p] = (8 * al + 6 * REF_PI * al * al + 8 * al * al * al) / C;
  wrap_particle(b, p);
  if (b->A[p] > b->Amax) b->Amax = b->A[p];
  if (b->R[p] > b->Rmax) b->Rmax = b->R[p];
}

/* calculate_packing_fraction, spherocyl_box.cpp:357-366 */
static double packing_fraction(const orc_box *b) {
  double filled = 0.0;
  for (int p = 0; p < b->n; p++) filled += (REF_PI * b->R[p] + 4.0 * b->A[p]) * b->R[p];
  return filled / (b->Lx * b->Ly);
}

/* ---- cell grid: configure_cells, spherocyl_box.cpp:223-268 ---- */
static int configure_cells(orc_box *b) {
  double wmin = (b->wfac > 0 ? b->wfac : 2.24) * (b->Rmax + b->Amax) + b->pad;
  double hmin = 2 * (b->Rmax + b->Amax) + b->pad;
  int rows = (int)(b->Ly / hmin);
  int cols = (int)(b->Lx / wmin);
  ivec_free_array(b->cells, b->ncells);
  free(b->cell_nbrs);
  b->rows = rows > 1 ? rows : 1;
  b->cols = cols > 1 ? cols : 1;
  b->ncells = b->rows * b->cols;
  b->W = b->Lx / b->cols;
  b->H = b->Ly / b->rows;
  if (b->pad == 0) {
    double dw = b->W - wmin, dh = b->H - hmin;
    b->pad = dw > dh ? dw : dh;
  }
  b->cells = (ivec *)calloc((size_t)b->ncells, sizeof(ivec));
  b->cell_nbrs = (int *)malloc((size_t)b->ncells * 8 * sizeof(int));
  if (!b->cells || !b->cell_nbrs) return -1;
  for (int c = 0; c < b->ncells; c++) {
    int row = c / b->cols, col = c % b->cols;
    int right = (col + 1) % b->cols, left = (b->cols + col - 1) % b->cols;
    int up = (row + 1) % b->rows, down = (b->rows + row - 1) % b->rows;
    int *t = b->cell_nbrs + 8 * c;
    /* table order of the reference: same row (+1, -1), row above (0, +1, -1),
     * row below (0, +1, -1) */
    t[0] = row * b->cols + right;
    t[1] = row * b->cols + left;
    t[2] = up * b->cols + col;
    t[3] = up * b->cols + right;
    t[4] = up * b->cols + left;
    t[5] = down * b->cols + col;
    t[6] = down * b->cols + right;
    t[7] = down * b->cols + left;
  }
  return 0;
}

/* find_cells, spherocyl_box.cpp:270-301 */
static void find_cells(orc_box *b) {
  for (int c = 0; c < b->ncells; c++) b->cells[c].len = 0;
  for (int p = 0; p < b->n; p++) {
    wrap_particle(b, p);
    int col = (int)(b->x[p] / b->W);
    int row = (int)(b->y[p] / b->H);
    /* A coordinate exactly equal to the box length survives the wrap and would
     * index one column/row past the grid in the reference; clamp it.  A
     * non-finite coordinate (crossing spines give 0/0 forces) is an error here,
     * where the reference would index out of bounds. */
    if (!isfinite(b->x[p]) || !isfinite(b->y[p])) b->err = 1;
    if (col >= b->cols || col < 0) col = col < 0 ? 0 : b->cols - 1;
    if (row >= b->rows || row < 0) row = row < 0 ? 0 : b->rows - 1;
    int c = col + row * b->cols;
    b->cell[p] = c;
    if (ivec_push(&b->cells[c], p)) b->err = 1;
  }
}

/* check_neighbors, spherocyl_box.cpp:303-318 */
static int check_neighbors(const orc_box *b, int p, int q) {
  double sig = b->R[p] + b->A[p] + b->R[q] + b->A[q];
  double dy = b->y[p] - b->y[q];
  dy += b->Ly * ((dy < -0.5 * b->Ly) - (dy > 0.5 * b->Ly));
  if (fabs(dy) < sig + b->pad) {
    double dx = b->x[p] - b->x[q];
    dx += b->Lx * ((dx < -0.5 * b->Lx) - (dx > 0.5 * b->Lx));
    double dxmax = dx + 0.5 * dy;
    dx += b->gamma * dy;
    if (fabs(dx) < sig + b->pad || fabs(dxmax) < sig + b->pad) return 1;
  }
  return 0;
}

/* find_neighbors, spherocyl_box.cpp:320-355 */
static void find_neighbors(orc_box *b) {
  b->n_rebuilds++;
  find_cells(b);
  for (int p = 0; p < b->n; p++) {
    b->nbrs[p].len = 0;
    b->xm[p] = 0.0;
    b->ym[p] = 0.0;
  }
  for (int p = 0; p < b->n - 1; p++) {
    int c = b->cell[p];
    for (int k = -1; k < 8; k++) {
      int cc = k < 0 ? c : b->cell_nbrs[8 * c + k];
      const ivec *cl = &b->cells[cc];
      for (int m = 0; m < cl->len; m++) {
        int q = cl->data[m];
        if (q > p && check_neighbors(b, p, q))
          if (ivec_push(&b->nbrs[p], q)) b->err = 1;
      }
    }
  }
}

/* ---- pair force.  calc_force_pair, strain_dynamics.cpp:17-75 (state copy),
 * calc_temp_force_pair :77-135 (predictor copy, gamma + dt*rate), and
 * calc_se_force_pair, spherocyl_box.cpp:425-500 (adds energy and stress). ---- */
typedef struct {
  const double *x, *y, *phi;
  double *fx, *fy, *tau;
} pview;

static void force_pair(orc_box *b, const pview *v, int p, int q, double gamma, double Lx, double Ly,
                       int with_se) {
  double dX = v->x[p] - v->x[q];
  double dY = v->y[p] - v->y[q];
  double phiP = v->phi[p], phiQ = v->phi[q];
  double sig = b->R[p] + b->R[q];
  double aP = b->A[p], aQ = b->A[q];
  dX += Lx * ((dX < -0.5 * Lx) - (dX > 0.5 * Lx));
  dY += Ly * ((dY < -0.5 * Ly) - (dY > 0.5 * Ly));
  dX += gamma * dY; /* sheared -> lab frame */

  double nxA = aP * cos(phiP), nyA = aP * sin(phiP);
  double nxB = aQ * cos(phiQ), nyB = aQ * sin(phiQ);
  double a = aP * aP;
  double bb = -(nxA * nxB + nyA * nyB);
  double c = aQ * aQ;
  double d = nxA * dX + nyA * dY;
  double e = -nxB * dX - nyB * dY;
  double delta = a * c - bb * bb;

  /* closest points of the two spines, clamped to the segments */
  double t = fmin(fmax((bb * d - a * e) / delta, -1.), 1.);
  double s = -(bb * t + d) / a;
  double sarg = fabs(s);
  s = fmin(fmax(s, -1.), 1.);
  if (sarg > 1) t = fmin(fmax(-(bb * s + e) / c, -1.), 1.);

  double dDx = dX + s * nxA - t * nxB;
  double dDy = dY + s * nyA - t * nyB;
  double dsq = dDx * dDx + dDy * dDy;
  if (dsq < sig * sig) {
    double dij = sqrt(dsq);
    double dvij = (1.0 - dij / sig) / sig;
    double Fx = dDx * dvij / dij;
    double Fy = dDy * dvij / dij;
    double tauP = s * nxA * Fy - s * nyA * Fx;
    double tauQ = t * nyB * Fx - t * nxB * Fy;
    v->fx[p] += Fx;
    v->fy[p] += Fy;
    v->tau[p] += tauP;
    v->fx[q] -= Fx;
    v->fy[q] -= Fy;
    v->tau[q] += tauQ;
    if (with_se) {
      /* stress arms and accumulation exactly as written in the reference,
       * including its three slips (spherocyl_box.cpp:486 uses nxB in the y arm,
       * :493 adds a Pxy term into Pxx, and Pyx is never reset by calc_se) */
      double CxA = s * nxA - 0.5 * dDx;
      double CyA = s * nyA - 0.5 * dDy;
      double CxB = t * nxB + 0.5 * dDx;
      double CyB = t * nxB + 0.5 * dDy;
      b->E += dvij * sig * (1.0 - dij / sig) / (2.0 * b->n);
      b->Pxx += Fx * CxA / (Lx * Ly);
      b->Pxx -= Fx * CxB / (Lx * Ly);
      b->Pyy += Fy * CyA / (Lx * Ly);
      b->Pyy -= Fy * CyB / (Lx * Ly);
      b->Pxy += Fy * CxA / (Lx * Ly);
      b->Pxx -= Fy * CxB / (Lx * Ly);
      b->Pyx += Fx * CyA / (Lx * Ly);
      b->Pyx -= Fx * CyB / (Lx * Ly);
    }
  }
}

/* ---- two-point contacts: euler_est_2p, src/cuda/2point_dynamics.cu:385-546.
 * PARITY UNPINNED: the reference implements this rule only in CUDA, which cannot
 * run here, so this restatement is checked only against its own invariants (forces
 * are the gradient of the summed contact energies) and the GPU kernels. ---- */
static void one_contact(orc_box *b, const pview *v, int p, int q, double dX, double dY, double s,
                        double t, double nxA, double nyA, double nxB, double nyB, double sig,
                        double Lx, double Ly, int with_se) {
  double dDx = dX + s * nxA - t * nxB;
  double dDy = dY + s * nyA - t * nyB;
  double dsq = dDx * dDx + dDy * dDy;
  if (!(dsq < sig * sig)) return;
  double dij = sqrt(dsq);
  double dvij = (1.0 - dij / sig) / sig;
  double Fx = dDx * dvij / dij, Fy = dDy * dvij / dij;
  v->fx[p] += Fx;
  v->fy[p] += Fy;
  v->tau[p] += s * nxA * Fy - s * nyA * Fx;
  v->fx[q] -= Fx;
  v->fy[q] -= Fy;
  v->tau[q] += t * nyB * Fx - t * nxB * Fy;
  if (with_se) {
    double LL = Lx * Ly;
    double CxA = s * nxA - 0.5 * dDx, CyA = s * nyA - 0.5 * dDy;
    double CxB = t * nxB + 0.5 * dDx, CyB = t * nyB + 0.5 * dDy;
    b->E += dvij * sig * (1.0 - dij / sig) / (2.0 * b->n);
    b->Pxx += Fx * CxA / LL - Fx * CxB / LL;
    b->Pyy += Fy * CyA / LL - Fy * CyB / LL;
    b->Pxy += Fy * CxA / LL - Fy * CxB / LL;
    b->Pyx += Fx * CyA / LL - Fx * CyB / LL;
  }
}

static double clamp1(double v) { return fmin(fmax(v, -1.0), 1.0); }

static void force_pair2(orc_box *b, const pview *v, int p, int q, double gamma, double Lx,
                        double Ly, int with_se) {
  double dX = v->x[p] - v->x[q], dY = v->y[p] - v->y[q];
  double sig = b->R[p] + b->R[q], aP = b->A[p], aQ = b->A[q];
  dX += Lx * ((dX < -0.5 * Lx) - (dX > 0.5 * Lx));
  dY += Ly * ((dY < -0.5 * Ly) - (dY > 0.5 * Ly));
  dX += gamma * dY;
  double nxA = aP * cos(v->phi[p]), nyA = aP * sin(v->phi[p]);
  double nxB = aQ * cos(v->phi[q]), nyB = aQ * sin(v->phi[q]);
  double a = aP * aP, bb = -(nxA * nxB + nyA * nyB), c = aQ * aQ;
  double d = nxA * dX + nyA * dY, e = -nxB * dX - nyB * dY;
  double delta = a * c - bb * bb;
  double s1, t1, s2, t2, s3, t3;
  if (delta <= 0) {
    /* parallel spines: the two ends of the overlap */
    s1 = clamp1(-(bb + d) / a);
    s2 = clamp1(-(d - bb) / a);
    if (fabs(s1) == 1)
      t1 = clamp1(-(bb * s1 + e) / c);
    else
      t1 = bb < 0 ? clamp1(-(bb + e) / c) : clamp1(-(e - bb) / c);
    if (fabs(s2) == 1)
      t2 = clamp1(-(bb * s2 + e) / c);
    else
      t2 = bb < 0 ? clamp1(-(e - bb) / c) : clamp1(-(bb + e) / c);
    s3 = s2;
    t3 = t2;
  } else {
    t1 = clamp1((bb * d - a * e) / delta);
    s1 = -(bb * t1 + d) / a;
    double sarg = fabs(s1);
    s1 = clamp1(s1);
    if (sarg >= 1) {
      /* primary contact at an end of A: the second candidate at A's other end */
      t1 = clamp1(-(bb * s1 + e) / c);
      s2 = -s1;
      t2 = -(bb * s2 + e) / c;
      double targ = fabs(t2);
      t2 = clamp1(t2);
      if (targ > 1) {
        s2 = clamp1(-(bb * t2 + d) / a);
        s3 = s2;
        t3 = t2;
      } else {
        t3 = bb < 0 ? -s1 : s1;
        s3 = -(bb * t3 + d) / a;
        sarg = fabs(s3);
        s3 = clamp1(s3);
        if (sarg >= 1) t3 = clamp1(-(bb * s3 + e) / c);
      }
    } else {
      /* primary contact at an end of B: the second candidate at B's other end */
      t2 = -t1;
      s2 = -(bb * t2 + d) / a;
      sarg = fabs(s2);
      s2 = clamp1(s2);
      if (sarg > 1) {
        t2 = clamp1(-(bb * s2 + e) / c);
        s3 = s2;
        t3 = t2;
      } else {
        s3 = bb < 0 ? -t1 : t1;
        t3 = -(bb * s3 + e) / c;
        double targ = fabs(t3);
        t3 = clamp1(t3);
        if (targ >= 1) s3 = clamp1(-(bb * t3 + d) / a);
      }
    }
  }
  one_contact(b, v, p, q, dX, dY, s1, t1, nxA, nyA, nxB, nyB, sig, Lx, Ly, with_se);
  if (s1 != s2 && t1 != t2) {
    if (s3 != s1 && s3 != s2) {
      double x2 = dX + s2 * nxA - t2 * nxB, y2 = dY + s2 * nyA - t2 * nyB;
      double x3 = dX + s3 * nxA - t3 * nxB, y3 = dY + s3 * nyA - t3 * nyB;
      if (x3 * x3 + y3 * y3 < x2 * x2 + y2 * y2) {
        s2 = s3;
        t2 = t3;
      }
    }
    one_contact(b, v, p, q, dX, dY, s2, t2, nxA, nyA, nxB, nyB, sig, Lx, Ly, with_se);
  }
}

void orc_set_two_point(orc_box *b, int on) { b->two_point = on != 0; }

static void zero3(double *a, double *b2, double *c, int n) {
  for (int i = 0; i < n; i++) {
    a[i] = 0.0;
    b2[i] = 0.0;
    c[i] = 0.0;
  }
}

static void loop_pairs(orc_box *b, const pview *v, double gamma, double Lx, double Ly, int with_se) {
  for (int p = 0; p < b->n; p++) {
    const ivec *nl = &b->nbrs[p];
    for (int j = 0; j < nl->len; j++) {
      int q = nl->data[j];
      if (q > p) {
        if (b->two_point)
          force_pair2(b, v, p, q, gamma, Lx, Ly, with_se);
        else
          force_pair(b, v, p, q, gamma, Lx, Ly, with_se);
      }
    }
  }
}

/* calc_forces, strain_dynamics.cpp:137-153 */
void orc_calc_forces(orc_box *b) {
  pview v = {b->x, b->y, b->phi, b->fx, b->fy, b->tau};
  zero3(b->fx, b->fy, b->tau, b->n);
  loop_pairs(b, &v, b->gamma, b->Lx, b->Ly, 0);
}

/* calc_temp_forces, strain_dynamics.cpp:156-172 (also what calc_resized_forces,
 * resize_dynamics.cpp:89-104, calls: the box lengths are the pre-resize ones) */
static void calc_temp_forces(orc_box *b) {
  pview v = {b->tx, b->ty, b->tphi, b->tfx, b->tfy, b->ttau};
  zero3(b->tfx, b->tfy, b->ttau, b->n);
  loop_pairs(b, &v, b->gamma + b->step * b->strain_rate, b->Lx, b->Ly, 0);
}

/* calc_se, spherocyl_box.cpp:502-522.  Pyx is deliberately not reset. */
void orc_calc_se(orc_box *b) {
  pview v = {b->x, b->y, b->phi, b->fx, b->fy, b->tau};
  zero3(b->fx, b->fy, b->tau, b->n);
  b->E = 0.0;
  b->Pxx = 0.0;
  b->Pyy = 0.0;
  b->Pxy = 0.0;
  loop_pairs(b, &v, b->gamma, b->Lx, b->Ly, 1);
}

void orc_zero_pyx(orc_box *b) { b->Pyx = 0.0; }

/* isolated_rotation, strain_dynamics.cpp:174-177 */
static double isolated_rotation(double RC, double phi) { return 0.5 * (1 - RC * cos(2 * phi)); }

static int moved_too_far(const orc_box *b, int i) {
  return b->xm[i] > 0.5 * b->pad || b->xm[i] < -0.5 * b->pad || b->ym[i] > 0.5 * b->pad ||
         b->ym[i] < -0.5 * b->pad;
}

/* set_back_gamma, spherocyl_box.cpp:524-545 */
static void set_back_gamma(orc_box *b) {
  for (int i = 0; i < b->n; i++) {
    if (b->y[i] < 0)
      b->y[i] += b->Ly;
    else if (b->y[i] > b->Ly)
      b->y[i] -= b->Ly;
    b->x[i] += b->y[i];
    if (b->x[i] < 0)
      b->x[i] += b->Lx;
    else {
      while (b->x[i] > b->Lx) b->x[i] -= b->Lx;
    }
  }
  b->gamma -= 1.0;
  b->gamma_total = (int)(b->gamma_total + 1) + b->gamma;
  find_neighbors(b);
}

/* strain_step, strain_dynamics.cpp:179-235 (Heun predictor-corrector under
 * Lees-Edwards shear, neighbour rebuild inside the corrector loop) */
int orc_strain_step(orc_box *b) {
  int n = b->n;
  double *fx0 = (double *)malloc(3 * (size_t)n * sizeof(double));
  if (!fx0) return -1;
  double *fy0 = fx0 + n, *tau0 = fy0 + n;
  for (int i = 0; i < n; i++) {
    fx0[i] = b->fx[i] - b->gamma * b->fy[i];
    fy0[i] = b->fy[i];
    tau0[i] = b->tau[i] / b->I[i] - b->strain_rate * isolated_rotation(b->RC[i], b->phi[i]);
    b->tx[i] = b->x[i] + b->step * fx0[i];
    b->ty[i] = b->y[i] + b->step * fy0[i];
    b->tphi[i] = b->phi[i] + b->step * tau0[i];
  }
  calc_temp_forces(b);
  for (int i = 0; i < n; i++) {
    double fx1 = b->tfx[i] - (b->gamma + b->step * b->strain_rate) * b->tfy[i];
    double fy1 = b->tfy[i];
    double tau1 = b->ttau[i] / b->I[i] - b->strain_rate * isolated_rotation(b->RC[i], b->tphi[i]);
    double ddx = 0.5 * b->step * (fx0[i] + fx1);
    double ddy = 0.5 * b->step * (fy0[i] + fy1);
    double ddphi = 0.5 * b->step * (tau0[i] + tau1);
    b->x[i] += ddx;
    b->y[i] += ddy;
    b->phi[i] += ddphi;
    b->xm[i] += ddx;
    b->ym[i] += ddy;
    if (moved_too_far(b, i)) find_neighbors(b);
  }
  free(fx0);
  b->gamma += b->strain_rate * b->step;
  b->gamma_total += b->strain_rate * b->step;
  if (b->gamma >= 0.5 && !b->no_setback) set_back_gamma(b);
  return b->err ? -1 : 0;
}

/* run_strain(dGammaMax), src/cuda/strain_dynamics.cu:1097-1108: cells for gamma up
 * to gamma_max, then strain steps (each followed by calc_forces) without set-back
 * until gamma >= gamma_max.  Returns the steps taken. */
long orc_strain_to_gamma(orc_box *b, double gamma_max) {
  double w = 2 * sqrt(gamma_max * gamma_max + 1);
  if (w > (b->wfac > 0 ? b->wfac : 2.24)) {
    b->wfac = w;
    if (configure_cells(b)) return -1;
    find_neighbors(b);
  }
  b->no_setback = 1;
  long k = 0;
  while (b->gamma < gamma_max) {
    if (orc_strain_step(b)) break;
    orc_calc_forces(b);
    k++;
  }
  b->no_setback = 0;
  return b->err ? -1 : k;
}

/* reconfigure_cells, resize_dynamics.cpp:106-121 (note the reference pairs the
 * row count with Lx and the column count with Ly; the boxes here are square) */
static void reconfigure_cells(orc_box *b) {
  double wmin = 2.24 * (b->Rmax + b->Amax) + b->pad;
  double hmin = 2 * (b->Rmax + b->Amax) + b->pad;
  int rows = (int)(b->Lx / hmin);
  int cols = (int)(b->Ly / wmin);
  if (rows < 1) rows = 1;
  if (cols < 1) cols = 1;
  if (rows != b->rows || cols != b->cols) {
    if (configure_cells(b)) b->err = 1;
    find_neighbors(b);
  } else {
    b->W = b->Lx / b->cols;
    b->H = b->Ly / b->rows;
  }
}

/* resize_step, resize_dynamics.cpp:164-243 (Heun at the set strain rate's gamma
 * with an affine scale of (1-rate)^dt applied to the predicted and corrected
 * positions; the box shrinks after the corrector loop) */
int orc_resize_step(orc_box *b, int shrink) {
  int n = b->n;
  double *fx0 = (double *)malloc(3 * (size_t)n * sizeof(double));
  if (!fx0) return -1;
  double *fy0 = fx0 + n, *tau0 = fy0 + n;
  for (int i = 0; i < n; i++) {
    fx0[i] = b->fx[i];
    fy0[i] = b->fy[i];
    tau0[i] = b->tau[i];
    b->tx[i] = b->x[i] + b->step * fx0[i];
    b->ty[i] = b->y[i] + b->step * fy0[i];
    b->tphi[i] = b->phi[i] + b->step * tau0[i] / b->I[i];
    if (shrink) {
      b->tx[i] *= pow(1.0 - b->resize_rate, b->step);
      b->ty[i] *= pow(1.0 - b->resize_rate, b->step);
    } else {
      b->tx[i] /= pow(1.0 - b->resize_rate, b->step);
      b->ty[i] /= pow(1.0 - b->resize_rate, b->step);
    }
  }
  calc_temp_forces(b);
  for (int i = 0; i < n; i++) {
    double ddx = 0.5 * b->step * (fx0[i] + b->tfx[i]);
    double ddy = 0.5 * b->step * (fy0[i] + b->tfy[i]);
    double ddphi = 0.5 * b->step * (tau0[i] + b->ttau[i]) / b->I[i];
    double x0 = b->x[i], y0 = b->y[i];
    b->x[i] += ddx;
    b->y[i] += ddy;
    b->phi[i] += ddphi;
    if (shrink) {
      b->x[i] *= pow(1.0 - b->resize_rate, b->step);
      b->y[i] *= pow(1.0 - b->resize_rate, b->step);
    } else {
      b->x[i] /= pow(1.0 - b->resize_rate, b->step);
      b->y[i] /= pow(1.0 - b->resize_rate, b->step);
    }
    b->xm[i] += b->x[i] - x0;
    b->ym[i] += b->y[i] - y0;
    reconfigure_cells(b);
    if (moved_too_far(b, i)) find_neighbors(b);
  }
  free(fx0);
  if (shrink) {
    b->Lx *= pow(1.0 - b->resize_rate, b->step);
    b->Ly *= pow(1.0 - b->resize_rate, b->step);
  } else {
    b->Lx /= pow(1.0 - b->resize_rate, b->step);
    b->Ly /= pow(1.0 - b->resize_rate, b->step);
  }
  return b->err ? -1 : 0;
}

/* pure_strain_step_2p, src/cuda/2point_dynamics.cu:2180-2283: predictor
 * pure_euler_est_2p :1872-1891 (the flow +x/2, -y/2 and the isolated rotation
 * -RC sin(2 phi)/2 at the strain rate, with the contact motion, by an Euler step),
 * corrector pure_heun_corr_2p :2140-2173 (forces at the predicted state in the
 * predicted box Lx(1 + dt rate/2) x Ly(1 - dt rate/2), gamma unchanged; the state
 * becomes the prediction plus dt/2 times the change of the contact motion), then
 * the box update :2255-2256, the total strain :2278, the grid check
 * (reconfigure_cells(0.0), src/cuda/spherocyl_box.cpp:46-67) and the rebuild.
 * Drag and rotation follow the src/cpp path: unit drag and the torque over I
 * (the src/cuda code divides by Kd times the area); the rebuild rule is the src/cpp
 * per-axis one, applied after the step as the src/cuda code does. */
int orc_pure_step(orc_box *b) {
  int n = b->n;
  double *f0 = (double *)malloc(3 * (size_t)n * sizeof(double));
  if (!f0) return -1;
  double *fx0 = f0, *fy0 = f0 + n, *tau0 = f0 + 2 * (size_t)n;
  const double e = b->strain_rate, dt = b->step;
  for (int i = 0; i < n; i++) {
    fx0[i] = b->fx[i];
    fy0[i] = b->fy[i];
    tau0[i] = b->tau[i];
    b->tx[i] = b->x[i] + dt * (b->fx[i] + 0.5 * e * b->x[i]);
    b->ty[i] = b->y[i] + dt * (b->fy[i] - 0.5 * e * b->y[i]);
    b->tphi[i] = b->phi[i] + dt * (b->tau[i] / b->I[i] + e * (-0.5 * b->RC[i] * sin(2 * b->phi[i])));
  }
  {
    pview v = {b->tx, b->ty, b->tphi, b->tfx, b->tfy, b->ttau};
    zero3(b->tfx, b->tfy, b->ttau, b->n);
    loop_pairs(b, &v, b->gamma, b->Lx * (1 + 0.5 * dt * e), b->Ly * (1 - 0.5 * dt * e), 0);
  }
  int rebuild = 0;
  for (int i = 0; i < n; i++) {
    double ddx = 0.5 * dt * (b->tfx[i] - fx0[i]);
    double ddy = 0.5 * dt * (b->tfy[i] - fy0[i]);
    double ddp = 0.5 * dt * (b->ttau[i] / b->I[i] - tau0[i] / b->I[i]);
    double x0 = b->x[i], y0 = b->y[i];
    b->x[i] = b->tx[i] + ddx;
    b->y[i] = b->ty[i] + ddy;
    b->phi[i] = b->tphi[i] + ddp;
    b->xm[i] += b->x[i] - x0;
    b->ym[i] += b->y[i] - y0;
    if (moved_too_far(b, i)) rebuild = 1;
  }
  free(f0);
  b->Lx += 0.5 * dt * e * b->Lx;
  b->Ly -= 0.5 * dt * e * b->Ly;
  b->gamma_total += dt * e;
  {
    double wmin = 2.24 * (b->Rmax + b->Amax) + b->pad;
    double hmin = 2 * (b->Rmax + b->Amax) + b->pad;
    int rows = (int)(b->Ly / hmin), cols = (int)(b->Lx / wmin);
    if (rows < 1) rows = 1;
    if (cols < 1) cols = 1;
    if (rows != b->rows || cols != b->cols) {
      if (configure_cells(b)) b->err = 1;
      rebuild = 1;
    } else {
      b->W = b->Lx / b->cols;
      b->H = b->Ly / b->rows;
    }
  }
  if (rebuild) find_neighbors(b);
  return b->err ? -1 : 0;
}

/* pure-shear steps, each followed by calc_forces (or calc_se when se_out) */
int orc_run_pure_steps(orc_box *b, int nsteps, double *se_out) {
  for (int k = 0; k < nsteps; k++) {
    if (orc_pure_step(b)) return -1;
    if (se_out) {
      orc_calc_se(b);
      orc_get_se(b, se_out + 5 * (size_t)k);
    } else {
      orc_calc_forces(b);
    }
  }
  return 0;
}

/* ---- Polak-Ribiere conjugate gradient: cjpr_relax_2p / cjpr_relax_step_2p /
 * line_search_2p, src/cuda/2point_dynamics.cu:3609-3780, 3886-4020, 4233-4296.
 * PARITY UNPINNED against the reference itself (its CG exists only in CUDA); the
 * GPU form is checked against this restatement.  The reference's norms are FP32
 * sums; here they are FP64.  Its line search is a recursion; this is the same
 * sequence of probes written as a loop, except that the reference's outer frame,
 * after a successful halving chain, also probes from the moved position: here a
 * line search ends with its move. ---- */

/* energy (calc_se's E) at x + t D */
static double probe_energy(orc_box *b, double t, const double *dx, const double *dy,
                           const double *dp) {
  for (int i = 0; i < b->n; i++) {
    b->tx[i] = b->x[i] + t * dx[i];
    b->ty[i] = b->y[i] + t * dy[i];
    b->tphi[i] = b->phi[i] + t * dp[i];
  }
  pview v = {b->tx, b->ty, b->tphi, b->tfx, b->tfy, b->ttau};
  zero3(b->tfx, b->tfy, b->ttau, b->n);
  b->E = 0.0;
  loop_pairs(b, &v, b->gamma, b->Lx, b->Ly, 1);
  return b->E;
}

enum { CG_TOP = 1, CG_SECOND, CG_HALVE, CG_DOUBLE, CG_FINAL, CG_MOVE, CG_FAIL };

/* line_search_2p from step0 in the current direction: 1 = moved, 0 = no lower
 * energy found (E0 is the energy at x) */
static int line_search(orc_box *b, double E0, double step, double min_step, double max_step,
                       const double *dx, const double *dy, const double *dp) {
  double E1 = 0, E2 = 0, tmin = 1;
  int phase = CG_TOP;
  double t = step;
  while (phase != CG_MOVE && phase != CG_FAIL) {
    double E = probe_energy(b, t, dx, dy, dp);
    int findmin = 0;
    switch (phase) {
      case CG_TOP:
        E1 = E;
        if (E1 > E0 && step > min_step) {
          step /= 2;
          E2 = E1;
          t = step;
          phase = CG_HALVE;
        } else {
          t = 2 * step;
          phase = CG_SECOND;
        }
        break;
      case CG_HALVE:
        E1 = E;
        if (E1 > E0 && step > min_step) {
          step /= 2;
          E2 = E1;
          t = step;
        } else {
          findmin = 1;
        }
        break;
      case CG_SECOND:
      case CG_DOUBLE:
        E2 = E;
        if (E2 <= E1 && step < max_step) {
          step *= 2;
          E1 = E2;
          t = 2 * step;
          phase = CG_DOUBLE;
        } else {
          findmin = 1;
        }
        break;
      case CG_FINAL:
        if (E > E1) tmin = 1;
        phase = CG_MOVE;
        break;
    }
    if (findmin) {
      if (E1 > E0) {
        phase = CG_FAIL;
      } else {
        tmin = (3 * E0 - 4 * E1 + E2) / (2 * E0 - 4 * E1 + 2 * E2);
        if (tmin > 2)
          tmin = 2;
        else if (E1 == E0)
          tmin = 1;
        t = tmin * step;
        phase = CG_FINAL;
      }
    }
  }
  if (phase == CG_FAIL) return 0;
  int rebuild = 0;
  const double h = tmin * step;
  for (int i = 0; i < b->n; i++) {
    double ddx = h * dx[i], ddy = h * dy[i];
    b->x[i] += ddx;
    b->y[i] += ddy;
    b->phi[i] += h * dp[i];
    b->xm[i] += ddx;
    b->ym[i] += ddy;
    if (moved_too_far(b, i)) rebuild = 1;
  }
  if (rebuild) find_neighbors(b);
  return 1;
}

/* Runs until a stop rule of cjpr_relax_step_2p holds or max_iter iterations; *iters,
 * *e_out (the calc_se energy at the last evaluation) and *reason (1 zero force,
 * 2 three equal energies, 3 no lower energy in any direction, 4 max_iter). */
int orc_cg_minimize(orc_box *b, int max_iter, int *iters, double *e_out, int *reason) {
  const int n = b->n;
  double *buf = (double *)calloc(6 * (size_t)n, sizeof(double));
  if (!buf) return -1;
  double *dx = buf, *dy = buf + n, *dp = buf + 2 * (size_t)n;
  double *f0x = buf + 3 * (size_t)n, *f0y = buf + 4 * (size_t)n, *f0p = buf + 5 * (size_t)n;
  double E0 = 0, Eh1 = 0, Eh2 = 0;
  int it = 0, why = 0;
  for (;;) {
    orc_calc_se(b);
    double F2 = 0, FF0 = 0, F02 = 0;
    for (int i = 0; i < n; i++) {
      F2 += b->fx[i] * b->fx[i] + b->fy[i] * b->fy[i] + b->tau[i] * b->tau[i];
      FF0 += b->fx[i] * f0x[i] + b->fy[i] * f0y[i] + b->tau[i] * f0p[i];
      F02 += f0x[i] * f0x[i] + f0y[i] * f0y[i] + f0p[i] * f0p[i];
    }
    Eh2 = Eh1;
    Eh1 = E0;
    E0 = b->E;
    if (F2 == 0) { why = 1; break; }
    if (Eh1 == E0 && Eh2 == Eh1) { why = 2; break; }
    if (it >= max_iter) { why = 4; break; }
    it++;
    int restart = (it - 1) % (3 * n) == 0;
    double beta = (restart || !(F02 > 0)) ? 0.0 : fmax(0.0, (F2 - FF0) / F02);
    for (int i = 0; i < n; i++) {
      dx[i] = b->fx[i] + beta * dx[i];
      dy[i] = b->fy[i] + beta * dy[i];
      dp[i] = b->tau[i] + beta * dp[i];
      f0x[i] = b->fx[i];
      f0y[i] = b->fy[i];
      f0p[i] = b->tau[i];
    }
    double norm = sqrt(F2 / (3 * n));
    double min_step = 1e-18 / norm, max_step = 2 / norm;
    if (line_search(b, E0, 2e-6 / norm, min_step, max_step, dx, dy, dp)) continue;
    /* steepest descent */
    for (int i = 0; i < n; i++) {
      dx[i] = b->fx[i];
      dy[i] = b->fy[i];
      dp[i] = b->tau[i];
    }
    if (line_search(b, E0, 1e-6 / norm, min_step, max_step, dx, dy, dp)) continue;
    /* F / sqrt|F| per particle (sqrt_grad_dir_2p, :3293-3340) */
    for (int i = 0; i < n; i++) {
      double fm = sqrt(b->fx[i] * b->fx[i] + b->fy[i] * b->fy[i]), tm = fabs(b->tau[i]);
      dx[i] = fm == 0 ? 0.0 : b->fx[i] / sqrt(fm);
      dy[i] = fm == 0 ? 0.0 : b->fy[i] / sqrt(fm);
      dp[i] = tm == 0 ? 0.0 : b->tau[i] / sqrt(tm);
    }
    double rn = sqrt(norm);
    if (line_search(b, E0, 2e-6 / rn, 1e-18 / rn, 2 / rn, dx, dy, dp)) continue;
    why = 3;
    break;
  }
  free(buf);
  if (iters) *iters = it;
  if (e_out) *e_out = E0;
  if (reason) *reason = why;
  return b->err ? -1 : 0;
}

/* gradient_relax_step, relaxation_dynamics.cpp:11-31 */
int orc_gd_step(orc_box *b) {
  for (int i = 0; i < b->n; i++) {
    double ddx = b->step * b->fx[i];
    double ddy = b->step * b->fy[i];
    b->x[i] += ddx;
    b->y[i] += ddy;
    b->phi[i] += b->step * b->tau[i] / b->I[i];
    b->xm[i] += ddx;
    b->ym[i] += ddy;
    if (moved_too_far(b, i)) find_neighbors(b);
  }
  return b->err ? -1 : 0;
}

/* ---- construction: SpherocylBox(L, N, x, y, phi, A*, R*, pad),
 * spherocyl_box.cpp:152-173 ---- */
orc_box *orc_create(int n, double L, const double *x, const double *y, const double *phi,
                    const double *A, const double *R, double pad) {
  return orc_create_rect(n, L, L, x, y, phi, A, R, pad);
}

/* The src/cuda box takes Lx and Ly (src/cuda/spherocyl_box.cpp:529-560); the
 * src/cpp routines used here already keep the two lengths apart. */
orc_box *orc_create_rect(int n, double Lx, double Ly, const double *x, const double *y,
                         const double *phi, const double *A, const double *R, double pad) {
  if (n <= 0 || !(Lx > 0) || !(Ly > 0)) return NULL;
  orc_box *b = (orc_box *)calloc(1, sizeof(orc_box));
  if (!b) return NULL;
  b->n = n;
  b->Lx = Lx;
  b->Ly = Ly;
  b->step = 0.05; /* set_defaults, spherocyl_box.cpp:16-53 */
  size_t nd = (size_t)n;
  double **arrs[] = {&b->x,  &b->y,   &b->phi, &b->R,  &b->A,  &b->I,   &b->RC, &b->fx, &b->fy,
                     &b->tau, &b->xm, &b->ym,  &b->tx, &b->ty, &b->tphi, &b->tfx, &b->tfy, &b->ttau};
  for (size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); k++) {
    *arrs[k] = (double *)calloc(nd, sizeof(double));
    if (!*arrs[k]) {
      orc_destroy(b);
      return NULL;
    }
  }
  b->cell = (int *)calloc(nd, sizeof(int));
  b->nbrs = (ivec *)calloc(nd, sizeof(ivec));
  if (!b->cell || !b->nbrs) {
    orc_destroy(b);
    return NULL;
  }
  for (int p = 0; p < n; p++) set_particle(b, p, x[p], y[p], phi[p], A[p], R[p]);
  b->packing = packing_fraction(b);
  b->pad = pad;
  if (configure_cells(b)) {
    orc_destroy(b);
    return NULL;
  }
  find_neighbors(b);
  return b;
}

void orc_destroy(orc_box *b) {
  if (!b) return;
  double *arrs[] = {b->x,  b->y,  b->phi, b->R,  b->A,  b->I,   b->RC,  b->fx,  b->fy,
                    b->tau, b->xm, b->ym, b->tx, b->ty, b->tphi, b->tfx, b->tfy, b->ttau};
  for (size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); k++) free(arrs[k]);
  free(b->cell);
  ivec_free_array(b->nbrs, b->n);
  ivec_free_array(b->cells, b->ncells);
  free(b->cell_nbrs);
  free(b);
}

/* setters mirror spherocyl_box.h:110-119 */
void orc_set_strain_rate(orc_box *b, double v) { b->strain_rate = v; }
void orc_set_resize_rate(orc_box *b, double v) { b->resize_rate = v; }
void orc_set_step(orc_box *b, double v) { b->step = v; }
void orc_set_gamma(orc_box *b, double v) { b->gamma = v; }
void orc_set_total_gamma(orc_box *b, double v) { b->gamma_total = v; }
void orc_find_neighbors(orc_box *b) { find_neighbors(b); }

int orc_n(const orc_box *b) { return b->n; }

void orc_get_state(const orc_box *b, double *x, double *y, double *phi) {
  memcpy(x, b->x, (size_t)b->n * sizeof(double));
  memcpy(y, b->y, (size_t)b->n * sizeof(double));
  memcpy(phi, b->phi, (size_t)b->n * sizeof(double));
}

void orc_get_forces(const orc_box *b, double *fx, double *fy, double *tau) {
  memcpy(fx, b->fx, (size_t)b->n * sizeof(double));
  memcpy(fy, b->fy, (size_t)b->n * sizeof(double));
  memcpy(tau, b->tau, (size_t)b->n * sizeof(double));
}

void orc_get_moved(const orc_box *b, double *xm, double *ym) {
  memcpy(xm, b->xm, (size_t)b->n * sizeof(double));
  memcpy(ym, b->ym, (size_t)b->n * sizeof(double));
}

void orc_get_consts(const orc_box *b, double *I, double *RC) {
  memcpy(I, b->I, (size_t)b->n * sizeof(double));
  memcpy(RC, b->RC, (size_t)b->n * sizeof(double));
}

/* out[0..9]: Lx Ly gamma gamma_total pad W H packing rows cols */
void orc_get_scalars(const orc_box *b, double *out) {
  out[0] = b->Lx;
  out[1] = b->Ly;
  out[2] = b->gamma;
  out[3] = b->gamma_total;
  out[4] = b->pad;
  out[5] = b->W;
  out[6] = b->H;
  out[7] = b->packing;
  out[8] = b->rows;
  out[9] = b->cols;
}

/* out[0..4]: E Pxx Pyy Pxy Pyx as the reference accumulates them */
void orc_get_se(const orc_box *b, double *out) {
  out[0] = b->E;
  out[1] = b->Pxx;
  out[2] = b->Pyy;
  out[3] = b->Pxy;
  out[4] = b->Pyx;
}

long orc_n_rebuilds(const orc_box *b) { return b->n_rebuilds; }

/* Number of half-list pairs; when pairs != NULL writes (p, q) pairs in list order. */
long orc_get_pairs(const orc_box *b, int *pairs, long cap) {
  long k = 0;
  for (int p = 0; p < b->n; p++) {
    for (int j = 0; j < b->nbrs[p].len; j++) {
      if (pairs && k < cap) {
        pairs[2 * k] = p;
        pairs[2 * k + 1] = b->nbrs[p].data[j];
      }
      k++;
    }
  }
  return k;
}

/* Inner loop of run_strain, strain_dynamics.cpp:285-296: strain_step followed by
 * calc_forces (or calc_se on stress-save steps).  se_out receives 5 values per
 * step when non-NULL (then calc_se runs every step). */
int orc_run_strain_steps(orc_box *b, int nsteps, double *se_out) {
  for (int k = 0; k < nsteps; k++) {
    if (orc_strain_step(b)) return -1;
    if (se_out) {
      orc_calc_se(b);
      orc_get_se(b, se_out + 5 * (size_t)k);
    } else {
      orc_calc_forces(b);
    }
  }
  return 0;
}

/* Inner loop of resize_box, resize_dynamics.cpp:297-307 */
int orc_run_resize_steps(orc_box *b, int nsteps, int shrink, double *se_out) {
  for (int k = 0; k < nsteps; k++) {
    if (orc_resize_step(b, shrink)) return -1;
    if (se_out) {
      orc_calc_se(b);
      orc_get_se(b, se_out + 5 * (size_t)k);
    } else {
      orc_calc_forces(b);
    }
  }
  return 0;
}

/* Loop body of gradient_descent_minimize, relaxation_dynamics.cpp:38-60
 * (calc_se, then a gradient step), without the file output.  Returns the number
 * of steps taken before E <= emin (or nsteps). */
int orc_run_gd_steps(orc_box *b, int nsteps, double emin, double *e_out) {
  int s;
  for (s = 0; s < nsteps; s++) {
    orc_calc_se(b);
    if (e_out) e_out[s] = b->E;
    if (b->E <= emin) break;
    if (orc_gd_step(b)) return -1;
  }
  return s;
}

/* ---- workload inputs: the seeded crossing-free packing ----
 *
 * The benchmark's reference arm runs the oracle on the same input packing as the
 * CUDA arm without loading the product library, so the generator of the inputs is
 * restated here: a SplitMix64 stream per seed, species alternating by index
 * (R_small, R_small * r_ratio, as src/cuda/spherocyl_box.cpp:1313-1314), A = a/R * R,
 * L from the packing fraction sum(pi R^2 + 4 A R)/L^2, and centres and angles
 * drawn uniformly with a placement redrawn while its spine comes closer than
 * min_sep (R_i + R_j) to an earlier spine (the reference's own rule,
 * check_particle_cross src/cpp/spherocyl_box.cpp:597-645, rejects only touching
 * spines and lets crossing-prone starts through; see the reference's 0/0 force
 * direction at src/cpp/strain_dynamics.cpp:58-62).  The draws and the rejection
 * test are the same floating-point operations as the library's generator, so the
 * two give the same packing bit for bit (tests/test_oracle_pin.py). */

static uint64_t sm64_next(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double sm64_uniform(uint64_t *s) {
  return (double)(sm64_next(s) >> 11) * (1.0 / 9007199254740992.0);
}

static double gen_cross(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

/* distance from a point to the segment c + t u, t in [-1, 1] */
static double gen_point_seg(double px, double py, double cx, double cy, double ux, double uy) {
  double uu = ux * ux + uy * uy;
  double t = 0.0;
  if (uu > 0) {
    t = ((px - cx) * ux + (py - cy) * uy) / uu;
    t = t < -1 ? -1 : (t > 1 ? 1 : t);
  }
  double dx = px - (cx + t * ux), dy = py - (cy + t * uy);
  return sqrt(dx * dx + dy * dy);
}

/* distance between the segments a + s u and b + t v: zero when they cross, else the
 * least endpoint-to-segment distance */
static double gen_seg_seg(double ax, double ay, double ux, double uy, double bx, double by,
                          double vx, double vy) {
  double p0x = ax - ux, p0y = ay - uy, p1x = ax + ux, p1y = ay + uy;
  double q0x = bx - vx, q0y = by - vy, q1x = bx + vx, q1y = by + vy;
  double d1 = gen_cross(q1x - q0x, q1y - q0y, p0x - q0x, p0y - q0y);
  double d2 = gen_cross(q1x - q0x, q1y - q0y, p1x - q0x, p1y - q0y);
  double d3 = gen_cross(p1x - p0x, p1y - p0y, q0x - p0x, q0y - p0y);
  double d4 = gen_cross(p1x - p0x, p1y - p0y, q1x - p0x, q1y - p0y);
  if (((d1 > 0 && d2 < 0) || (d1 < 0 && d2 > 0)) && ((d3 > 0 && d4 < 0) || (d3 < 0 && d4 > 0)))
    return 0.0;
  double m = gen_point_seg(p0x, p0y, bx, by, vx, vy);
  m = fmin(m, gen_point_seg(p1x, p1y, bx, by, vx, vy));
  m = fmin(m, gen_point_seg(q0x, q0y, ax, ay, ux, uy));
  m = fmin(m, gen_point_seg(q1x, q1y, ax, ay, ux, uy));
  return m;
}

int orc_generate_packing(int n, double packing, double a_over_r, double r_small, double r_ratio,
                         uint64_t seed, double min_sep, double *x, double *y, double *phi,
                         double *R, double *A, double *L_out) {
  if (n < 2 || !(packing > 0 && packing < 1) || !(a_over_r >= 0) || !(r_small > 0) ||
      !(r_ratio > 0) || !(min_sep >= 0) || !x || !y || !phi || !R || !A || !L_out)
    return 1;
  const double pi = 3.14159265358979323846;
  double filled = 0.0, rmax = 0.0, amax = 0.0;
  for (int i = 0; i < n; i++) {
    R[i] = (i % 2 == 0) ? r_small : r_small * r_ratio;
    A[i] = a_over_r * R[i];
    filled += pi * R[i] * R[i] + 4.0 * A[i] * R[i];
    rmax = fmax(rmax, R[i]);
    amax = fmax(amax, A[i]);
  }
  const double L = sqrt(filled / packing);
  *L_out = L;
  /* bins of at least the reach: two spines closer than min_sep (R_i + R_j) have
   * centres within 2 A_max + 2 min_sep R_max; a bin list is a linked list */
  const double reach = 2.0 * amax + 2.0 * min_sep * rmax;
  int ng = (int)(L / fmax(reach, 1e-300));
  if (ng > 2048) ng = 2048;
  const int gridded = ng >= 3;
  if (!gridded) ng = 1;
  const double gw = L / ng;
  int *head = (int *)malloc((size_t)ng * ng * sizeof(int));
  int *next = (int *)malloc((size_t)n * sizeof(int));
  if (!head || !next) {
    free(head);
    free(next);
    return 2;
  }
  for (long c = 0; c < (long)ng * ng; c++) head[c] = -1;
  uint64_t rng = seed * 0x2545F4914F6CDD1Dull + 0x1234567ull;
  const long max_tries = 1000000;
  int rc = 0;
  for (int i = 0; i < n && rc == 0; i++) {
    long tries = 0;
    for (;;) {
      if (++tries > max_tries) {
        rc = 3;
        break;
      }
      double xi = L * sm64_uniform(&rng), yi = L * sm64_uniform(&rng);
      double pi_ = pi * sm64_uniform(&rng);
      double ux = A[i] * cos(pi_), uy = A[i] * sin(pi_);
      int gx = gridded ? (int)(xi / gw) : 0, gy = gridded ? (int)(yi / gw) : 0;
      if (gx > ng - 1) gx = ng - 1;
      if (gy > ng - 1) gy = ng - 1;
      int ok = 1, span = gridded ? 1 : 0;
      for (int a = -span; a <= span && ok; a++)
        for (int b = -span; b <= span && ok; b++) {
          int cx = (gx + b + ng) % ng, cy = (gy + a + ng) % ng;
          for (int j = head[(long)cy * ng + cx]; j >= 0; j = next[j]) {
            double dx = xi - x[j], dy = yi - y[j];
            dx -= L * round(dx / L);
            dy -= L * round(dy / L);
            double vx = A[j] * cos(phi[j]), vy = A[j] * sin(phi[j]);
            if (gen_seg_seg(dx, dy, ux, uy, 0.0, 0.0, vx, vy) < min_sep * (R[i] + R[j])) {
              ok = 0;
              break;
            }
          }
        }
      if (!ok) continue;
      x[i] = xi;
      y[i] = yi;
      phi[i] = pi_;
      long c = (long)gy * ng + gx;
      next[i] = head[c];
      head[c] = i;
      break;
    }
  }
  free(head);
  free(next);
  return rc;
}
