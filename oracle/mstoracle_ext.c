/* Oracle extensions beyond the reference (test infrastructure only; see
 * mstoracle.h).  The reference has no limiter, no CFL or local time step,
 * no Runge-Kutta update and no periodic faces, and its 2nd-order outlet
 * and symmetry faces are broken (RhoSolver.cpp:320-361); these functions
 * restate the methods the CUDA path implements for them, in the kernels'
 * operation order.  Compile with -ffp-contract=off. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mstoracle.h"

void om_default_params_ext(om_params_ext *p) {
  memset(p, 0, sizeof *p);
  p->flux = OM_AUSM;
  p->order = 1;
  p->quirks = 1;
  p->dt = 1.0 / 4e+3;
  p->cfl = 0.5;
  om_reference_inlet(p->inlet_q);
  p->viscous = 0;
  p->mu = 1.7894e-05;
  p->lam = -0.666667 * 1.7894e-05;
  p->kappa = 0.0242;
  p->cv = 715.8;
}

/* Laminar viscous term, the intent of RhoSolver::updateViscid
 * (RhoSolver.cpp:371-429) with its defects corrected: primitive gradients
 * from the conserved cell gradients by the chain rule, eta0-weighted face
 * values and gradients, tau = mu (grad u + grad u^T) + lambda (div u) I,
 * energy u.tau + kappa grad T (T = e / cv); no-slip adiabatic walls with the
 * velocity gradient corrected along the cell-to-face vector. */
static void prim_grad_e(const double q[4], const double g[8], double cv, double gu[2],
                        double gv[2], double gT[2]) {
  const double rho = q[0], u = q[1] / rho, v = q[2] / rho, er = q[3] / rho;
  for (int d = 0; d < 2; ++d) {
    gu[d] = (g[4 * d + 1] - u * g[4 * d]) / rho;
    gv[d] = (g[4 * d + 2] - v * g[4 * d]) / rho;
    const double ge = (g[4 * d + 3] - er * g[4 * d]) / rho - u * gu[d] - v * gv[d];
    gT[d] = ge / cv;
  }
}
static void sub_viscous_e(double u, double v, const double gu[2], const double gv[2],
                          const double gT[2], double mu, double lam, double kappa, int heat,
                          double F[8]) {
  const double div = gu[0] + gv[1];
  const double txx = mu * (2.0 * gu[0]) + lam * div;
  const double tyy = mu * (2.0 * gv[1]) + lam * div;
  const double txy = mu * (gu[1] + gv[0]);
  const double qx = heat ? kappa * gT[0] : 0.0;
  const double qy = heat ? kappa * gT[1] : 0.0;
  F[1] = F[1] - txx;
  F[2] = F[2] - txy;
  F[3] = F[3] - ((u * txx + v * txy) + qx);
  F[5] = F[5] - txy;
  F[6] = F[6] - tyy;
  F[7] = F[7] - ((u * txy + v * tyy) + qy);
}

static double shift(const om_mesh *m, int f, int d) {
  return m->face_shift ? m->face_shift[2 * f + d] : 0.0;
}

/* Green-Gauss gradient of conserved Q from eta0-weighted face values
 * (RhoSolver.cpp:430-453).  quirks = 1 copies c0 values from face nInt-1
 * on (the reference's boundary loop); 0 from nInt. */
void om_gradient_ext(const om_mesh *m, const double *q, int quirks,
                     double *grad) {
  const int first = quirks ? (m->n_int_faces > 0 ? m->n_int_faces - 1 : 0)
                           : m->n_int_faces;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < m->n_cells; ++c) {
    double g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const int f = m->cell_faces[k];
      const int c0 = m->face_cells[2 * f], c1 = m->face_cells[2 * f + 1];
      double fq[4];
      if (f < first && c1 >= 0) {
        const double e = m->face_eta0[f];
        for (int j = 0; j < 4; ++j) fq[j] = e * q[4 * c0 + j] + (1 - e) * q[4 * c1 + j];
      } else {
        for (int j = 0; j < 4; ++j) fq[j] = q[4 * c0 + j];
      }
      for (int j = 0; j < 4; ++j) g[j] += fq[j] * m->cell_dof[2 * k];
      for (int j = 0; j < 4; ++j) g[4 + j] += fq[j] * m->cell_dof[2 * k + 1];
    }
    for (int j = 0; j < 8; ++j) grad[8 * c + j] = g[j] / m->cell_vol[c];
  }
}

static void mirror_e(double dx, double dy, const double in[4], double out[4]) {
  const double nrm = sqrt(dx * dx + dy * dy);
  const double n0 = dx / nrm, n1 = dy / nrm;
  double t = n0 * in[1];
  t += n1 * in[2];
  out[0] = in[0];
  out[1] = in[1] - 2.0 * n0 * t;
  out[2] = in[2] - 2.0 * n1 * t;
  out[3] = in[3];
}

static void recon_e(const double q[4], const double *g, double rx, double ry,
                    double out[4]) {
  for (int k = 0; k < 4; ++k) {
    double s = g[k] * rx;
    s += g[4 + k] * ry;
    out[k] = q[k] + s;
  }
}

/* TVD slope limiters psi(a, b) of the upwind difference a and the central
 * difference b: minmod; van Leer 2ab/(a+b); van Albada
 * (a(b^2+e) + b(a^2+e)) / (a^2+b^2+2e), e = 1e-12 (van Albada, van Leer &
 * Roberts 1982); zero unless a and b have the same sign. */
static double slope_e(int lim, double a, double b) {
  if (!(a * b > 0.0)) return 0.0;
  if (lim == OM_LIM_MINMOD) return fabs(a) < fabs(b) ? a : b;
  if (lim == OM_LIM_VANLEER) return 2.0 * a * b / (a + b);
  const double e = 1e-12;
  return (a * (b * b + e) + b * (a * a + e)) / (a * a + b * b + 2.0 * e);
}

/* Face flux matrices with the extended options.  quirks = 1 is identical to
 * om_face_flux.  quirks = 0: left/right from the geometry (c0 is left along
 * axis d when its outward normal points +d), 2nd-order symmetry faces
 * mirror the reconstructed state, 2nd-order outlets use the reconstructed
 * state on both sides.  With a limiter (quirks = 0), interior faces use the
 * edge-based MUSCL reconstruction Q_L = Q_0 + psi(2 G_0.d - dQ, dQ)/2,
 * Q_R = Q_1 - psi(2 G_1.d - dQ, dQ)/2 with d = x_1 - x_0 (periodic image)
 * and dQ = Q_1 - Q_0, which reduces to 1D MUSCL on a uniform grid; boundary
 * faces are first order. */
void om_face_flux_ext(const om_mesh *m, const om_params_ext *p,
                      const double *q, const double *grad, double *F) {
  void (*fl)(const double *, const double *, int, double *) =
      (p->flux == OM_ROE) ? om_roe_flux : om_ausm_flux;
  const int second = (p->order == 2);
  const int limited = second && !p->quirks && p->limiter != OM_LIM_NONE;
  for (int z = 0; z < m->n_zones; ++z) {
    const int type = m->zone[4 * z + 3];
#pragma omp parallel for schedule(static)
    for (int i = m->zone[4 * z + 1] - 1; i < m->zone[4 * z + 2]; ++i) {
      double *Fi = F + 8 * i;
      const int c0 = m->face_cells[2 * i], c1 = m->face_cells[2 * i + 1];
      const double *dv = m->face_dir + 2 * i;
      int flag[2];
      for (int d = 0; d < 2; ++d)
        flag[d] = p->quirks ? m->face_flag[2 * i + d] : (m->face_dac[i] * dv[d] >= 0);
      if (type != 2 && type != 3 && type != 5 && type != 7 && type != 10) {
        memset(Fi, 0, 8 * sizeof(double));
        continue;
      }
      const double *q0 = q + 4 * c0;
      double r0x = 0, r0y = 0;
      if (second) {
        r0x = m->face_ctr[2 * i] - m->cell_ctr[2 * c0];
        r0y = m->face_ctr[2 * i + 1] - m->cell_ctr[2 * c0 + 1];
      }
      double L[4], R[4];
      if (type == 2) {
        const double *q1 = q + 4 * c1;
        if (!second) {
          memcpy(L, q0, 32);
          memcpy(R, q1, 32);
        } else {
          const double r1x = (m->face_ctr[2 * i] - shift(m, i, 0)) - m->cell_ctr[2 * c1];
          const double r1y = (m->face_ctr[2 * i + 1] - shift(m, i, 1)) - m->cell_ctr[2 * c1 + 1];
          const double *g0 = grad + 8 * c0, *g1 = grad + 8 * c1;
          if (!limited) {
            recon_e(q0, g0, r0x, r0y, L);
            recon_e(q1, g1, r1x, r1y, R);
          } else {
            const double dx = r0x - r1x, dy = r0y - r1y;
            double *ph = p->phi ? p->phi + 8 * (size_t)i : NULL;
            for (int k = 0; k < 4; ++k) {
              const double dc = q1[k] - q0[k];
              const double du0 = 2.0 * (g0[k] * dx + g0[4 + k] * dy) - dc;
              const double du1 = 2.0 * (g1[k] * dx + g1[4 + k] * dy) - dc;
              if (ph && p->phi_mode == 2) {
                /* frozen limiter: the recorded ratios times the current
                 * upwind differences (a smooth reconstruction) */
                L[k] = q0[k] + 0.5 * (ph[k] * du0);
                R[k] = q1[k] - 0.5 * (ph[4 + k] * du1);
                continue;
              }
              const double s0 = slope_e(p->limiter, du0, dc);
              const double s1 = slope_e(p->limiter, du1, dc);
              L[k] = q0[k] + 0.5 * s0;
              R[k] = q1[k] - 0.5 * s1;
              if (ph && p->phi_mode == 1) {
                ph[k] = du0 != 0.0 ? s0 / du0 : 0.0;
                ph[4 + k] = du1 != 0.0 ? s1 / du1 : 0.0;
              }
            }
            if (p->positivity) {
              /* a side whose reconstructed density or pressure is not
               * positive falls back to its cell value */
              const double pl = (L[3] - 0.5 * (L[1] * L[1] + L[2] * L[2]) / L[0]) * (1.4 - 1.0);
              const double pr = (R[3] - 0.5 * (R[1] * R[1] + R[2] * R[2]) / R[0]) * (1.4 - 1.0);
              if (!(L[0] > 0.0) || !(pl > 0.0)) memcpy(L, q0, 32);
              if (!(R[0] > 0.0) || !(pr > 0.0)) memcpy(R, q1, 32);
            }
          }
        }
      } else {
        const int recon_side = second && !limited && !(type == 7 && p->quirks) &&
                               !(type == 5 && p->quirks);
        if (recon_side) recon_e(q0, grad + 8 * c0, r0x, r0y, L);
        else memcpy(L, q0, 32);
        if (type == 10) {
          memcpy(R, p->inlet_q, 32);
        } else if (type == 5) {
          memcpy(R, L, 32);
        } else if (type == 3 && second && p->viscous) {
          R[0] = L[0];
          R[1] = -L[1];
          R[2] = -L[2];
          R[3] = L[3];
        } else if (type == 7 && second && p->quirks && !limited) {
          double rc[4], mm[4];
          recon_e(q0, grad + 8 * c0, r0x, r0y, rc);
          mirror_e(dv[0], dv[1], q0, mm);
          R[0] = rc[0];
          R[1] = mm[1];
          R[2] = mm[2];
          R[3] = rc[3];
        } else {
          mirror_e(dv[0], dv[1], L, R);
        }
      }
      for (int d = 0; d < 2; ++d) {
        if (flag[d]) fl(L, R, d, Fi + 4 * d);
        else fl(R, L, d, Fi + 4 * d);
      }
      if (second && p->viscous && (type == 2 || type == 3)) {
        double gu[2], gv[2], gT[2];
        prim_grad_e(q0, grad + 8 * c0, p->cv, gu, gv, gT);
        if (type == 2) {
          const double *q1 = q + 4 * c1;
          const double eta = m->face_eta0[i], ome = 1.0 - eta;
          double gu1[2], gv1[2], gT1[2], qf[4];
          prim_grad_e(q1, grad + 8 * c1, p->cv, gu1, gv1, gT1);
          for (int d = 0; d < 2; ++d) {
            gu[d] = eta * gu[d] + ome * gu1[d];
            gv[d] = eta * gv[d] + ome * gv1[d];
            gT[d] = eta * gT[d] + ome * gT1[d];
          }
          for (int k = 0; k < 4; ++k) qf[k] = eta * q0[k] + ome * q1[k];
          sub_viscous_e(qf[1] / qf[0], qf[2] / qf[0], gu, gv, gT, p->mu, p->lam, p->kappa, 1, Fi);
        } else {
          const double rl = sqrt(r0x * r0x + r0y * r0y);
          const double ex = r0x / rl, ey = r0y / rl;
          const double u0 = q0[1] / q0[0], v0 = q0[2] / q0[0];
          const double cu = (0.0 - u0) / rl - (gu[0] * ex + gu[1] * ey);
          const double cvv = (0.0 - v0) / rl - (gv[0] * ex + gv[1] * ey);
          gu[0] = gu[0] + cu * ex;
          gu[1] = gu[1] + cu * ey;
          gv[0] = gv[0] + cvv * ex;
          gv[1] = gv[1] + cvv * ey;
          sub_viscous_e(0.0, 0.0, gu, gv, gT, p->mu, p->lam, p->kappa, 0, Fi);
        }
      }
    }
  }
}

double om_spectral_dt(const om_mesh *m, const double *q, double cfl,
                      double *dt_cell) {
  double dmin = 1e300;
#pragma omp parallel for schedule(static) reduction(min : dmin)
  for (int c = 0; c < m->n_cells; ++c) {
    const double *qs = q + 4 * c;
    const double u = qs[1] / qs[0], v = qs[2] / qs[0];
    const double ke = 0.5 * (qs[1] * qs[1] + qs[2] * qs[2]) / qs[0];
    const double pr = (qs[3] - ke) * (1.4 - 1);
    const double snd = sqrt(1.4 * pr / qs[0]);
    double lam = 0.0;
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const double *dv = m->face_dir + 2 * m->cell_faces[k];
      lam += fabs(u * dv[0] + v * dv[1]) + snd * sqrt(dv[0] * dv[0] + dv[1] * dv[1]);
    }
    double dtc = cfl * m->cell_vol[c] / (0.5 * lam);
    if (!(dtc > 0)) dtc = 0.0;
    if (dt_cell) dt_cell[c] = dtc;
    if (dtc < dmin) dmin = dtc;
  }
  return dmin;
}

/* residual R(q) of every cell with the extended options */
static void residual_ext(const om_mesh *m, const om_params_ext *p,
                         const double *q, double *F, double *grad, double *R) {
  if (p->order == 2) om_gradient_ext(m, q, p->quirks, grad);
  om_face_flux_ext(m, p, q, grad, F);
  om_gather(m, F, R);
}

int om_step_ext(const om_mesh *m, const om_params_ext *p, double *q,
                int nsteps, double t_end, double *time, om_norms *last) {
  const int nC = m->n_cells;
  double *F = (double *)calloc((size_t)8 * m->n_faces, 8);
  double *grad = (double *)calloc((size_t)8 * nC, 8);
  double *R = (double *)calloc((size_t)4 * nC, 8);
  double *q1 = (double *)calloc((size_t)4 * nC, 8);
  double *qn = (double *)calloc((size_t)4 * nC, 8);
  double *dtc = (double *)calloc((size_t)nC, 8);
  if (!F || !grad || !R || !q1 || !qn || !dtc) {
    free(F), free(grad), free(R), free(q1), free(qn), free(dtc);
    return OM_EINVAL;
  }
  double t = time ? *time : 0.0;
  for (int s = 0; s < nsteps; ++s) {
    if (t_end > 0 && t >= t_end) break; /* further steps would have dt = 0 */
    double dt = p->dt;
    if (p->dt_mode != OM_DT_FIXED) dt = om_spectral_dt(m, q, p->cfl, dtc);
    if (t_end > 0 && t + dt > t_end) dt = t_end - t;
    if (dt < 0) dt = 0;
    const int local = (p->dt_mode == OM_DT_CFL_LOCAL);
    const double *qin = q;
    double *out = p->rk2 ? q1 : qn;
    residual_ext(m, p, q, F, grad, R);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nC; ++c) {
      const double f = (local ? dtc[c] : dt) / m->cell_vol[c];
      for (int j = 0; j < 4; ++j) out[4 * c + j] = q[4 * c + j] - f * R[4 * c + j];
    }
    if (p->rk2) {
      qin = q1;
      residual_ext(m, p, q1, F, grad, R);
#pragma omp parallel for schedule(static)
      for (int c = 0; c < nC; ++c) {
        const double f = (local ? dtc[c] : dt) / m->cell_vol[c];
        for (int j = 0; j < 4; ++j)
          qn[4 * c + j] = 0.5 * q[4 * c + j] + 0.5 * (q1[4 * c + j] - f * R[4 * c + j]);
      }
    }
    if (last) {
      memset(last, 0, sizeof *last);
      for (int c = 0; c < nC; ++c) {
        const double v = m->cell_vol[c];
        for (int j = 0; j < 4; ++j) {
          const double ch = fabs(qn[4 * c + j] - qin[4 * c + j]) / qin[4 * c + j];
          if (last->linf[j] < ch) last->linf[j] = ch;
          const double rv = R[4 * c + j] / v;
          last->l2[j] += rv * rv;
        }
        last->mass += v * qn[4 * c];
      }
      for (int j = 0; j < 4; ++j) last->l2[j] = sqrt(last->l2[j] / (double)nC);
      last->dt = dt;
    }
    t += dt;
    memcpy(q, qn, sizeof(double) * 4 * nC);
  }
  if (last) last->time = t;
  if (time) *time = t;
  free(F), free(grad), free(R), free(q1), free(qn), free(dtc);
  return OM_OK;
}
