// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A C-ABI shim around the reference's own CPU classes (tmarschall/spherocyls
// src/cpp), compiled from the reference sources where they lie by oracle/Makefile
// into oracle/_ref/.  It reaches the per-step routines of SpherocylBox
// (strain_step, calc_forces, calc_se, resize_step, gradient_relax_step, the
// particle array and the neighbour lists) so that the tests can pin the oracle
// (spherocyl_oracle.c) against the reference itself, step by step, without the
// reference's file output.  Nothing here is part of the product library.
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

// The per-step routines and the particle state are private members of the
// reference class; open them for this shim only.
#define private public
#include "spherocyl_box.h"
#undef private

namespace {
struct Silence {
  // The reference prints cell-grid chatter on stdout from configure_cells.
  Silence() { std::cout.rdbuf(nullptr); }
} silence_stdout;
}  // namespace

extern "C" {

void *ref_create(int n, double L, const double *x, const double *y, const double *phi,
                 const double *A, const double *R, double pad) {
  std::vector<double> vx(x, x + n), vy(y, y + n), vp(phi, phi + n), va(A, A + n), vr(R, R + n);
  // SpherocylBox(L, N, x, y, phi, A*, R*, pad): src/cpp/spherocyl_box.cpp:152-173
  SpherocylBox *b = new SpherocylBox(L, n, vx.data(), vy.data(), vp.data(), va.data(), vr.data(), pad);
  b->m_dPyx = 0.0;  // never initialised by the reference (spherocyl_box.cpp:34-37)
  return b;
}

void ref_destroy(void *h) { delete static_cast<SpherocylBox *>(h); }

void ref_set_params(void *h, double strain_rate, double resize_rate, double step, double gamma,
                    double total_gamma) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  b->set_strain_rate(strain_rate);
  b->set_resize_rate(resize_rate);
  b->set_step(step);
  b->set_gamma(gamma);
  b->set_total_gamma(total_gamma);
}

void ref_find_neighbors(void *h) { static_cast<SpherocylBox *>(h)->find_neighbors(); }
void ref_calc_forces(void *h) { static_cast<SpherocylBox *>(h)->calc_forces(); }
void ref_calc_se(void *h) { static_cast<SpherocylBox *>(h)->calc_se(); }
void ref_strain_step(void *h) { static_cast<SpherocylBox *>(h)->strain_step(); }
void ref_resize_step(void *h, int shrink) { static_cast<SpherocylBox *>(h)->resize_step(shrink != 0); }
void ref_gd_step(void *h) { static_cast<SpherocylBox *>(h)->gradient_relax_step(); }

int ref_n(void *h) { return static_cast<SpherocylBox *>(h)->m_nParticles; }

void ref_get_state(void *h, double *x, double *y, double *phi) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  for (int p = 0; p < b->m_nParticles; p++) {
    x[p] = b->m_psParticles[p].m_dX;
    y[p] = b->m_psParticles[p].m_dY;
    phi[p] = b->m_psParticles[p].m_dPhi;
  }
}

void ref_get_forces(void *h, double *fx, double *fy, double *tau) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  for (int p = 0; p < b->m_nParticles; p++) {
    fx[p] = b->m_psParticles[p].m_dFx;
    fy[p] = b->m_psParticles[p].m_dFy;
    tau[p] = b->m_psParticles[p].m_dTau;
  }
}

void ref_get_moved(void *h, double *xm, double *ym) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  for (int p = 0; p < b->m_nParticles; p++) {
    xm[p] = b->m_psParticles[p].m_dXMoved;
    ym[p] = b->m_psParticles[p].m_dYMoved;
  }
}

void ref_get_consts(void *h, double *I, double *RC) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  for (int p = 0; p < b->m_nParticles; p++) {
    I[p] = b->m_psParticles[p].m_dI;
    RC[p] = b->m_psParticles[p].m_dRC;
  }
}

void ref_get_scalars(void *h, double *out) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  out[0] = b->m_dLx;
  out[1] = b->m_dLy;
  out[2] = b->m_dGamma;
  out[3] = b->m_dGammaTotal;
  out[4] = b->m_dPadding;
  out[5] = b->m_dCellWidth;
  out[6] = b->m_dCellHeight;
  out[7] = b->m_dPacking;
  out[8] = b->m_nCellRows;
  out[9] = b->m_nCellCols;
}

void ref_get_se(void *h, double *out) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  out[0] = b->m_dEnergy;
  out[1] = b->m_dPxx;
  out[2] = b->m_dPyy;
  out[3] = b->m_dPxy;
  out[4] = b->m_dPyx;
}

long ref_get_pairs(void *h, int *pairs, long cap) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  long k = 0;
  for (int p = 0; p < b->m_nParticles; p++) {
    for (size_t j = 0; j < b->m_pvNeighbors[p].size(); j++) {
      if (pairs && k < cap) {
        pairs[2 * k] = p;
        pairs[2 * k + 1] = b->m_pvNeighbors[p][j];
      }
      k++;
    }
  }
  return k;
}

// The inner loop of run_strain (src/cpp/strain_dynamics.cpp:285-296) without
// file output: strain_step, then calc_se (when se_out) or calc_forces.
int ref_run_strain_steps(void *h, int nsteps, double *se_out) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  for (int k = 0; k < nsteps; k++) {
    b->strain_step();
    if (se_out) {
      b->calc_se();
      ref_get_se(h, se_out + 5 * static_cast<size_t>(k));
    } else {
      b->calc_forces();
    }
  }
  return 0;
}

// The inner loop of resize_box (src/cpp/resize_dynamics.cpp:297-307).
int ref_run_resize_steps(void *h, int nsteps, int shrink, double *se_out) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  for (int k = 0; k < nsteps; k++) {
    b->resize_step(shrink != 0);
    if (se_out) {
      b->calc_se();
      ref_get_se(h, se_out + 5 * static_cast<size_t>(k));
    } else {
      b->calc_forces();
    }
  }
  return 0;
}

// The loop of gradient_descent_minimize (src/cpp/relaxation_dynamics.cpp:38-60)
// without file output.
int ref_run_gd_steps(void *h, int nsteps, double emin, double *e_out) {
  SpherocylBox *b = static_cast<SpherocylBox *>(h);
  int s;
  for (s = 0; s < nsteps; s++) {
    b->calc_se();
    if (e_out) e_out[s] = b->m_dEnergy;
    if (b->m_dEnergy <= emin) break;
    b->gradient_relax_step();
  }
  return s;
}

}  // extern "C"
