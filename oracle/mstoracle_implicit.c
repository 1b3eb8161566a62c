/* CPU restatement of the project's implicit steady iterations (matrix-free
 * LU-SGS on colour groups) for the density-based path.
 *
 * TEST INFRASTRUCTURE ONLY (see mstoracle.h): the checker of the product's
 * batched implicit solver (mst_batch_*).  The reference has no implicit
 * density-based solver (its lusolver serves the pressure-based path), so
 * this is a restatement of the project's own algorithm -- Yoon and
 * Jameson's LU-SGS, AIAA J. 26(9), 1988 -- on the oracle's residual
 * (om_gradient_ext, om_face_flux_ext, om_gather in corrected mode), with
 * every operation in the order the CUDA kernels evaluate it (compiled with
 * -ffp-contract=off; the parity kernels without FMA), so one iteration
 * agrees bit-for-bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mstoracle.h"
#include "mstoracle_implicit.h"

static const double kGm1 = 1.4 - 1.0;
static const double kGamma = 1.4;
static const double kViscSpectral = 1.4 / 0.72;

static double lambda_of(const double *q, double sx, double sy, double area,
                        double vol, double mu, int viscous) {
  const double ir = 1.0 / q[0];
  const double u = q[1] * ir, v = q[2] * ir;
  const double p = kGm1 * (q[3] - 0.5 * (q[1] * u + q[2] * v));
  const double a = sqrt(kGamma * p * ir);
  double lam = fabs(u * sx + v * sy) + a * area;
  if (viscous) lam += 2.0 * kViscSpectral * mu * ir * area * area / vol;
  return lam;
}

static void flux_diff(const double *q, const double *dq, double sx, double sy,
                      double *out) {
  double fa[4], fb[4], w[4];
  int k;
  {
    const double ir = 1.0 / q[0];
    const double un = (q[1] * sx + q[2] * sy) * ir;
    const double p = kGm1 * (q[3] - 0.5 * (q[1] * q[1] + q[2] * q[2]) * ir);
    fa[0] = q[0] * un;
    fa[1] = q[1] * un + p * sx;
    fa[2] = q[2] * un + p * sy;
    fa[3] = (q[3] + p) * un;
  }
  for (k = 0; k < 4; ++k) w[k] = q[k] + dq[k];
  {
    const double ir = 1.0 / w[0];
    const double un = (w[1] * sx + w[2] * sy) * ir;
    const double p = kGm1 * (w[3] - 0.5 * (w[1] * w[1] + w[2] * w[2]) * ir);
    fb[0] = w[0] * un;
    fb[1] = w[1] * un + p * sx;
    fb[2] = w[2] * un + p * sy;
    fb[3] = (w[3] + p) * un;
  }
  for (k = 0; k < 4; ++k) out[k] = fb[k] - fa[k];
}

/* off-diagonal sum of cell c over neighbours of lower (fwd) or higher
 * colour, and (fwd) the diagonal's Lambda */
static void offdiag(const om_mesh *m, const double *q, const double *dq,
                    const int *color, int c, int fwd, double mu, int viscous,
                    double omega, double *off, double *lam_sum) {
  const int col = color[c];
  double lam = 0.0;
  int k, j;
  for (j = 0; j < 4; ++j) off[j] = 0.0;
  for (k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
    const int f = m->cell_faces[k];
    const double sx = m->cell_dof[2 * k], sy = m->cell_dof[2 * k + 1];
    const double area = sqrt(sx * sx + sy * sy);
    int nb, cj;
    if (fwd) lam += lambda_of(q + 4 * (size_t)c, sx, sy, area, m->cell_vol[c], mu, viscous);
    if (m->face_cells[2 * f + 1] < 0) continue; /* boundary face */
    nb = m->cell_nb[k];
    cj = color[nb];
    if (fwd ? !(cj < col) : !(cj > col)) continue;
    {
      double fd[4];
      const double *qj = q + 4 * (size_t)nb, *dqj = dq + 4 * (size_t)nb;
      double lj;
      flux_diff(qj, dqj, sx, sy, fd);
      lj = omega * lambda_of(qj, sx, sy, area, m->cell_vol[nb], mu, viscous);
      for (j = 0; j < 4; ++j) off[j] += 0.5 * (fd[j] - lj * dqj[j]);
    }
  }
  if (lam_sum) *lam_sum = lam;
}

int om_lusgs_iterate(const om_mesh *m, const om_params_ext *p, double *q,
                     const int *color, const om_lusgs_params *ip, int niter,
                     double *l2_hist) {
  const int nC = m->n_cells;
  double *F = (double *)calloc((size_t)8 * (m->n_faces > 0 ? m->n_faces : 1), 8);
  double *grad = (double *)calloc((size_t)8 * nC, 8);
  double *R = (double *)calloc((size_t)4 * nC, 8);
  double *dq = (double *)calloc((size_t)4 * nC, 8);
  double *D = (double *)calloc((size_t)nC, 8);
  double *qn = (double *)calloc((size_t)4 * nC, 8);
  double first = 0.0, cfl = ip->cfl0;
  int it, c, j, ncol = 0, col;
  if (!F || !grad || !R || !dq || !D || !qn) {
    free(F), free(grad), free(R), free(dq), free(D), free(qn);
    return OM_EINVAL;
  }
  for (c = 0; c < nC; ++c) ncol = color[c] + 1 > ncol ? color[c] + 1 : ncol;
  om_params_ext pp = *p;
  pp.positivity = 1;
  double *phi = NULL;
  int frozen = 0; /* 0 live limiter, 1 record this iteration, 2 frozen */
  int converged = 0;
  double l2_win = 0.0, frz_best = 0.0;
  int frz_best_it = 0;
  if (ip->freeze_tol > 0) {
    phi = (double *)calloc((size_t)8 * (m->n_faces > 0 ? m->n_faces : 1), 8);
    pp.phi = phi;
  }
  double l2_conv = 0.0;
  for (it = 0; it < niter; ++it) {
    double s = 0.0, l2;
    if (converged) {
      /* nothing of a converged case runs again: its state and norms stay */
      if (l2_hist) l2_hist[it] = l2_conv;
      continue;
    }
    pp.phi_mode = phi ? frozen : 0;
    if (p->order == 2) om_gradient_ext(m, q, 0, grad);
    om_face_flux_ext(m, &pp, q, p->order == 2 ? grad : NULL, F);
    om_gather(m, F, R);
    for (c = 0; c < nC; ++c) {
      const double x = R[4 * (size_t)c] / m->cell_vol[c];
      s += x * x;
    }
    l2 = sqrt(s / (double)(nC > 0 ? nC : 1));
    if (it == 0) first = l2;
    if (l2_hist) l2_hist[it] = l2;
    /* limiter freezing: the iteration after the case first falls below
     * freeze_tol records the limiter ratios, later ones reuse them */
    if (frozen == 1) {
      frozen = 2;
      frz_best = l2;
      frz_best_it = it;
    } else if (phi && frozen == 0 && it > 0 && it % 50 == 0) {
      /* freeze once stagnating below freeze_tol: L2 fell by less than 30%
       * over the last 50 iterations */
      if (first > 0.0 && l2 <= ip->freeze_tol * first && l2 > 0.7 * l2_win) frozen = 1;
      l2_win = l2;
    } else if (frozen == 2 && ip->refreeze_window > 0) {
      /* re-freeze: no new best (below 0.9 of it) for refreeze_window
       * iterations records the ratios again from the current state */
      if (l2 < 0.9 * frz_best) {
        frz_best = l2;
        frz_best_it = it;
      } else if (it - frz_best_it >= ip->refreeze_window) {
        frozen = 1;
      }
    }
    if (ip->tol > 0 && first > 0.0 && l2 <= ip->tol * first) {
      converged = 1; /* the state that met the tolerance is kept */
      l2_conv = l2;
      continue;
    }
    /* the CFL of this iteration from the norms of this residual */
    cfl = ip->cfl0;
    if (l2 > 0.0 && first > 0.0) cfl = ip->cfl0 * (first / l2);
    cfl = cfl < ip->cfl0 ? ip->cfl0 : cfl;
    cfl = cfl > ip->cfl_max ? ip->cfl_max : cfl;
    if (!(cfl == cfl)) cfl = ip->cfl0;
    for (col = 0; col < ncol; ++col)
      for (c = 0; c < nC; ++c) {
        double off[4], lam, d;
        if (color[c] != col) continue;
        offdiag(m, q, dq, color, c, 1, p->mu, p->viscous, ip->omega, off, &lam);
        d = lam * (1.0 / cfl + 0.5 * ip->omega);
        D[c] = d;
        for (j = 0; j < 4; ++j) dq[4 * (size_t)c + j] = -(R[4 * (size_t)c + j] + off[j]) / d;
      }
    for (col = ncol - 1; col >= 0; --col)
      for (c = 0; c < nC; ++c) {
        double off[4];
        if (color[c] != col) continue;
        offdiag(m, q, dq, color, c, 0, p->mu, p->viscous, ip->omega, off, NULL);
        for (j = 0; j < 4; ++j) dq[4 * (size_t)c + j] = dq[4 * (size_t)c + j] - off[j] / D[c];
        {
          /* positivity: halve the update (at most 6 times, else drop it)
           * until density and pressure stay above a fifth of their values */
          const double *qc = q + 4 * (size_t)c, *dc = dq + 4 * (size_t)c;
          const double p0 = kGm1 * (qc[3] - 0.5 * (qc[1] * qc[1] + qc[2] * qc[2]) / qc[0]);
          double alpha = 1.0, n[4];
          int ok = 0, h;
          for (h = 0; h < 7 && !ok; ++h) {
            double pn;
            for (j = 0; j < 4; ++j) n[j] = qc[j] + alpha * dc[j];
            pn = kGm1 * (n[3] - 0.5 * (n[1] * n[1] + n[2] * n[2]) / n[0]);
            ok = n[0] > 0.2 * qc[0] && pn > 0.2 * p0;
            if (!ok) alpha *= 0.5;
          }
          for (j = 0; j < 4; ++j) qn[4 * (size_t)c + j] = ok ? n[j] : qc[j];
          if (ip->p_floor > 0.0) {
            double *w = qn + 4 * (size_t)c;
            const double ke = 0.5 * (w[1] * w[1] + w[2] * w[2]) / w[0];
            const double pw = kGm1 * (w[3] - ke);
            if (pw < ip->p_floor * w[0]) w[3] = ke + ip->p_floor * w[0] / kGm1;
          }
        }
      }
    memcpy(q, qn, sizeof(double) * 4 * (size_t)nC);
  }
  free(F), free(grad), free(R), free(dq), free(D), free(qn), free(phi);
  return OM_OK;
}

/* Greedy colouring in file cell order: each cell takes the smallest colour
 * none of its (interior-face) neighbours holds.  Returns the colour count. */
int om_greedy_colors(const om_mesh *m, int *color) {
  int c, k, ncol = 0;
  for (c = 0; c < m->n_cells; ++c) color[c] = -1;
  for (c = 0; c < m->n_cells; ++c) {
    unsigned used = 0;
    int pick = 0;
    for (k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const int f = m->cell_faces[k];
      if (m->face_cells[2 * f + 1] < 0) continue;
      {
        const int nb = m->cell_nb[k];
        if (nb != c && color[nb] >= 0 && color[nb] < 32) used |= 1u << color[nb];
      }
    }
    while (used & (1u << pick)) ++pick;
    color[c] = pick;
    if (pick + 1 > ncol) ncol = pick + 1;
  }
  return ncol;
}
