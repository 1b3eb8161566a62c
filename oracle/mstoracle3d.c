/* CPU restatement of the 3D density-based residual path (test
 * infrastructure only; see mstoracle3d.h for what it restates and why).
 * Compile with -ffp-contract=off: every operation is rounded in the order
 * written, which is the order of the CUDA exact path. */
#include "mstoracle3d.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double kGamma = 1.4;
#define GM1 (1.4 - 1.0)

static double dot3(const double *a, const double *b) {
  double s = a[0] * b[0];
  s += a[1] * b[1];
  s += a[2] * b[2];
  return s;
}

void om3_free(om3_mesh *m) {
  free(m->face_cells), free(m->face_kind), free(m->face_ctr), free(m->face_dir);
  free(m->r0), free(m->r1), free(m->eta), free(m->cell_ctr), free(m->cell_vol);
  free(m->cell_ptr), free(m->cell_faces), free(m->cell_nb), free(m->cell_dir);
  free(m->cell_w);
  memset(m, 0, sizeof *m);
}

static int kind_of(int type, int c1) {
  switch (type) {
    case 2: return c1 >= 0 ? 0 : 5;
    case 10: return 1;
    case 3: return 2;
    case 7: return 3;
    case 5: return 4;
    default: return 5;
  }
}

int om3_build(const om3_input *in, om3_mesh *m) {
  const int nF = in->n_faces, nC = in->n_cells;
  int f, c, k, d;
  memset(m, 0, sizeof *m);
  m->n_cells = nC;
  m->n_faces = nF;
  m->face_cells = (int *)malloc(sizeof(int) * 2 * (size_t)nF);
  m->face_kind = (int *)malloc(sizeof(int) * (size_t)nF);
  m->face_ctr = (double *)malloc(sizeof(double) * 3 * (size_t)nF);
  m->face_dir = (double *)malloc(sizeof(double) * 3 * (size_t)nF);
  m->r0 = (double *)calloc(3 * (size_t)nF, sizeof(double));
  m->r1 = (double *)calloc(3 * (size_t)nF, sizeof(double));
  m->eta = (double *)malloc(sizeof(double) * (size_t)nF);
  m->cell_ctr = (double *)calloc(3 * (size_t)nC, sizeof(double));
  m->cell_vol = (double *)calloc((size_t)nC, sizeof(double));
  m->cell_ptr = (int *)calloc((size_t)nC + 1, sizeof(int));
  if (!m->face_cells || !m->face_kind || !m->face_ctr || !m->face_dir || !m->r0 || !m->r1 ||
      !m->eta || !m->cell_ctr || !m->cell_vol || !m->cell_ptr) {
    om3_free(m);
    return 1;
  }
  for (f = 0; f < nF; ++f) {
    const int c0 = in->face_cells[2 * f], c1 = in->face_cells[2 * f + 1];
    const int b = in->face_ptr[f], n = in->face_ptr[f + 1] - b;
    const double *p0 = in->node_xyz + 3 * (size_t)in->face_nodes[b];
    const double *p1 = in->node_xyz + 3 * (size_t)in->face_nodes[b + 1];
    const double *p2 = in->node_xyz + 3 * (size_t)in->face_nodes[b + 2];
    double a[3], bb[3];
    if (c0 < 0 || c0 >= nC || c1 >= nC || (n != 3 && n != 4)) {
      om3_free(m);
      return 1;
    }
    m->face_cells[2 * f] = c0;
    m->face_cells[2 * f + 1] = c1;
    m->face_kind[f] = kind_of(in->face_type[f], c1);
    for (d = 0; d < 3; ++d) {
      double s = p0[d];
      s += p1[d];
      s += p2[d];
      if (n == 4) s += in->node_xyz[3 * (size_t)in->face_nodes[b + 3] + d];
      m->face_ctr[3 * f + d] = s / (double)n;
    }
    if (n == 3) {
      for (d = 0; d < 3; ++d) {
        a[d] = p1[d] - p0[d];
        bb[d] = p2[d] - p0[d];
      }
    } else {
      const double *p3 = in->node_xyz + 3 * (size_t)in->face_nodes[b + 3];
      for (d = 0; d < 3; ++d) {
        a[d] = p2[d] - p0[d];
        bb[d] = p3[d] - p1[d];
      }
    }
    m->face_dir[3 * f] = 0.5 * (a[1] * bb[2] - a[2] * bb[1]);
    m->face_dir[3 * f + 1] = 0.5 * (a[2] * bb[0] - a[0] * bb[2]);
    m->face_dir[3 * f + 2] = 0.5 * (a[0] * bb[1] - a[1] * bb[0]);
    m->cell_ptr[c0 + 1]++;
    if (c1 >= 0) m->cell_ptr[c1 + 1]++;
  }
  for (c = 0; c < nC; ++c) m->cell_ptr[c + 1] += m->cell_ptr[c];
  {
    const int tot = m->cell_ptr[nC];
    int *fill = (int *)malloc(sizeof(int) * ((size_t)nC + 1));
    m->cell_faces = (int *)malloc(sizeof(int) * (size_t)(tot > 0 ? tot : 1));
    m->cell_nb = (int *)malloc(sizeof(int) * (size_t)(tot > 0 ? tot : 1));
    m->cell_dir = (double *)malloc(sizeof(double) * 3 * (size_t)(tot > 0 ? tot : 1));
    m->cell_w = (double *)malloc(sizeof(double) * 2 * (size_t)(tot > 0 ? tot : 1));
    if (!fill || !m->cell_faces || !m->cell_nb || !m->cell_dir || !m->cell_w) {
      free(fill);
      om3_free(m);
      return 1;
    }
    memcpy(fill, m->cell_ptr, sizeof(int) * (size_t)nC);
    for (f = 0; f < nF; ++f) {
      const int c0 = m->face_cells[2 * f], c1 = m->face_cells[2 * f + 1];
      m->cell_faces[fill[c0]] = f;
      m->cell_nb[fill[c0]++] = c1;
      if (c1 >= 0) {
        m->cell_faces[fill[c1]] = f;
        m->cell_nb[fill[c1]++] = c0;
      }
    }
    free(fill);
  }
  /* cell centre = mean of the face centres in the cell's own frame */
  for (c = 0; c < nC; ++c) {
    const int kb = m->cell_ptr[c], ke = m->cell_ptr[c + 1];
    double s[3] = {0.0, 0.0, 0.0};
    for (k = kb; k < ke; ++k) {
      const int ff = m->cell_faces[k];
      const int own = m->face_cells[2 * ff] == c;
      for (d = 0; d < 3; ++d) {
        double x = m->face_ctr[3 * ff + d];
        if (!own && in->c1_shift) x = x - in->c1_shift[3 * ff + d];
        s[d] += x;
      }
    }
    for (d = 0; d < 3; ++d) m->cell_ctr[3 * c + d] = s[d] / (double)(ke - kb);
  }
  /* orientation out of c0, reconstruction offsets, eta0 */
  for (f = 0; f < nF; ++f) {
    const int c0 = m->face_cells[2 * f], c1 = m->face_cells[2 * f + 1];
    double t[3];
    for (d = 0; d < 3; ++d) t[d] = m->face_ctr[3 * f + d] - m->cell_ctr[3 * c0 + d];
    if (dot3(m->face_dir + 3 * f, t) < 0.0)
      for (d = 0; d < 3; ++d) m->face_dir[3 * f + d] = -m->face_dir[3 * f + d];
    for (d = 0; d < 3; ++d) m->r0[3 * f + d] = t[d];
    m->eta[f] = 1.0;
    if (c1 >= 0) {
      double n0, n1;
      for (d = 0; d < 3; ++d) {
        double x = m->face_ctr[3 * f + d];
        if (in->c1_shift) x = x - in->c1_shift[3 * f + d];
        m->r1[3 * f + d] = x - m->cell_ctr[3 * c1 + d];
      }
      n0 = sqrt(dot3(m->r0 + 3 * f, m->r0 + 3 * f));
      n1 = sqrt(dot3(m->r1 + 3 * f, m->r1 + 3 * f));
      m->eta[f] = n1 / (n0 + n1);
    }
  }
  /* per cell-face outward area vector and weights; volume by the
   * divergence theorem, V = 1/3 sum (x_f - x_c) . S_out */
  for (c = 0; c < nC; ++c) {
    double v = 0.0;
    for (k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const int ff = m->cell_faces[k];
      const int own = m->face_cells[2 * ff] == c;
      const double *r = own ? m->r0 + 3 * ff : m->r1 + 3 * ff;
      for (d = 0; d < 3; ++d)
        m->cell_dir[3 * k + d] = own ? m->face_dir[3 * ff + d] : -m->face_dir[3 * ff + d];
      m->cell_w[2 * k] = own ? m->eta[ff] : 1.0 - m->eta[ff];
      m->cell_w[2 * k + 1] = own ? 1.0 - m->eta[ff] : m->eta[ff];
      v += dot3(r, m->cell_dir + 3 * k);
    }
    m->cell_vol[c] = v / 3.0;
  }
  return 0;
}

void om3_gradient(const om3_mesh *m, const double *q, double *grad) {
  int c, k, j;
  for (c = 0; c < m->n_cells; ++c) {
    const double *qs = q + 5 * (size_t)c;
    double g[15];
    const double vol = m->cell_vol[c];
    for (j = 0; j < 15; ++j) g[j] = 0.0;
    for (k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const int nb = m->cell_nb[k];
      const double *dv = m->cell_dir + 3 * k;
      double fq[5];
      if (nb < 0) {
        for (j = 0; j < 5; ++j) fq[j] = qs[j];
      } else {
        const double w0 = m->cell_w[2 * k], w1 = m->cell_w[2 * k + 1];
        const double *qn = q + 5 * (size_t)nb;
        for (j = 0; j < 5; ++j) fq[j] = w0 * qs[j] + w1 * qn[j];
      }
      for (j = 0; j < 5; ++j) g[j] += fq[j] * dv[0];
      for (j = 0; j < 5; ++j) g[5 + j] += fq[j] * dv[1];
      for (j = 0; j < 5; ++j) g[10 + j] += fq[j] * dv[2];
    }
    for (j = 0; j < 15; ++j) grad[15 * (size_t)c + j] = g[j] / vol;
  }
}

static double p_of(const double q[5]) {
  const double ke = 0.5 * ((q[1] * q[1] + q[2] * q[2]) + q[3] * q[3]) / q[0];
  return (q[4] - ke) * GM1;
}

static double entropy_fix(double x) {
  const double e = 0.125;
  if (x > e) return x;
  return (x * x + e * e) / 2.0 / e;
}

/* 1D Roe flux along axis d between l (left) and r (right) */
static void roe3(const double l[5], const double r[5], int d, double f[5]) {
  const double D = sqrt(fabs(r[0] / l[0]));
  double u[3], du[3], FL[5], FR[5], dis[5];
  int k;
  for (k = 0; k < 3; ++k) u[k] = (l[k + 1] / l[0] + D * r[k + 1] / r[0]) / (1.0 + D);
  const double pL = p_of(l), pR = p_of(r);
  const double hL = (l[4] + pL) / l[0], hR = (r[4] + pR) / r[0];
  const double H = (hL + D * hR) / (1.0 + D);
  const double uu = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2];
  const double a = sqrt(fabs(GM1 * (H - 0.5 * uu)));
  const double ud = u[d];
  const double l1 = entropy_fix(fabs(ud - a)), l2 = entropy_fix(fabs(ud)),
               l5 = entropy_fix(fabs(ud + a));
  const double rt = D * l[0];
  const double drho = r[0] - l[0], dp = pR - pL;
  for (k = 0; k < 3; ++k) du[k] = r[k + 1] / r[0] - l[k + 1] / l[0];
  const double a2 = a * a;
  const double al1 = (dp - rt * a * du[d]) / (2.0 * a2);
  const double al5 = (dp + rt * a * du[d]) / (2.0 * a2);
  const double al2 = drho - dp / a2;
  const double w1 = l1 * al1, w2 = l2 * al2, w5 = l5 * al5, ws = l2 * rt;
  FL[0] = l[d + 1];
  FR[0] = r[d + 1];
  for (k = 0; k < 3; ++k) {
    FL[1 + k] = l[d + 1] * l[k + 1] / l[0];
    FR[1 + k] = r[d + 1] * r[k + 1] / r[0];
  }
  FL[1 + d] = FL[1 + d] + pL;
  FR[1 + d] = FR[1 + d] + pR;
  FL[4] = hL * l[d + 1];
  FR[4] = hR * r[d + 1];
  dis[0] = (w1 + w2) + w5;
  {
    double sh = 0.0;
    for (k = 0; k < 3; ++k) {
      const double ak = (k == d) ? a : 0.0;
      double s = (w1 * (u[k] - ak) + w2 * u[k]) + w5 * (u[k] + ak);
      if (k != d) {
        s += ws * du[k];
        sh += u[k] * du[k];
      }
      dis[1 + k] = s;
    }
    dis[4] = ((w1 * (H - ud * a) + w2 * (0.5 * uu)) + w5 * (H + ud * a)) + ws * sh;
  }
  for (k = 0; k < 5; ++k) f[k] = 0.5 * (FL[k] + FR[k]) - 0.5 * dis[k];
}

static double slope3(int lim, double a, double b) {
  if (!(a * b > 0.0)) return 0.0;
  if (lim == 1) return fabs(a) < fabs(b) ? a : b;
  if (lim == 2) return 2.0 * a * b / (a + b);
  {
    const double e = 1e-12;
    return (a * (b * b + e) + b * (a * a + e)) / (a * a + b * b + 2.0 * e);
  }
}

static void recon3(const double q[5], const double *g, const double *r, double out[5]) {
  int k;
  for (k = 0; k < 5; ++k) {
    double s = g[k] * r[0];
    s += g[5 + k] * r[1];
    s += g[10 + k] * r[2];
    out[k] = q[k] + s;
  }
}

static void mirror3(const double *dv, const double in[5], double out[5]) {
  const double nrm = sqrt((dv[0] * dv[0] + dv[1] * dv[1]) + dv[2] * dv[2]);
  const double n0 = dv[0] / nrm, n1 = dv[1] / nrm, n2 = dv[2] / nrm;
  double t = n0 * in[1];
  t += n1 * in[2];
  t += n2 * in[3];
  out[0] = in[0];
  out[1] = in[1] - 2.0 * n0 * t;
  out[2] = in[2] - 2.0 * n1 * t;
  out[3] = in[3] - 2.0 * n2 * t;
  out[4] = in[4];
}

static void prim_grad3(const double q[5], const double *g, double cv, double gu[3],
                       double gv[3], double gw[3], double gT[3]) {
  const double rho = q[0], u = q[1] / rho, v = q[2] / rho, w = q[3] / rho, er = q[4] / rho;
  int d;
  for (d = 0; d < 3; ++d) {
    const double *gd = g + 5 * d;
    gu[d] = (gd[1] - u * gd[0]) / rho;
    gv[d] = (gd[2] - v * gd[0]) / rho;
    gw[d] = (gd[3] - w * gd[0]) / rho;
    {
      const double ge = (gd[4] - er * gd[0]) / rho - u * gu[d] - v * gv[d] - w * gw[d];
      gT[d] = ge / cv;
    }
  }
}

static void sub_viscous3(double u, double v, double w, const double gu[3], const double gv[3],
                         const double gw[3], const double gT[3], double mu, double lam,
                         double kappa, int heat, double *F) {
  const double div = (gu[0] + gv[1]) + gw[2];
  double t[3][3];
  int d;
  t[0][0] = mu * (2.0 * gu[0]) + lam * div;
  t[1][1] = mu * (2.0 * gv[1]) + lam * div;
  t[2][2] = mu * (2.0 * gw[2]) + lam * div;
  t[0][1] = t[1][0] = mu * (gu[1] + gv[0]);
  t[0][2] = t[2][0] = mu * (gu[2] + gw[0]);
  t[1][2] = t[2][1] = mu * (gv[2] + gw[1]);
  for (d = 0; d < 3; ++d) {
    const double qd = heat ? kappa * gT[d] : 0.0;
    double *Fd = F + 5 * d;
    Fd[1] = Fd[1] - t[0][d];
    Fd[2] = Fd[2] - t[1][d];
    Fd[3] = Fd[3] - t[2][d];
    Fd[4] = Fd[4] - (((u * t[0][d] + v * t[1][d]) + w * t[2][d]) + qd);
  }
}

static void face_flux3(const om3_mesh *m, const om3_params *p, const double *q,
                       const double *grad, int f, double F[15]) {
  const int kind = m->face_kind[f];
  const int c0 = m->face_cells[2 * f], c1 = m->face_cells[2 * f + 1];
  const double *dv = m->face_dir + 3 * f;
  const int second = p->order == 2 && grad != NULL;
  const int limited = second && p->limiter != 0;
  const double *q0 = q + 5 * (size_t)c0, *g0 = second ? grad + 15 * (size_t)c0 : NULL;
  const double *q1 = NULL, *g1 = NULL;
  double L[5], R[5];
  int k, d;
  if (kind == 5) {
    for (k = 0; k < 15; ++k) F[k] = 0.0;
    return;
  }
  if (kind == 0) {
    q1 = q + 5 * (size_t)c1;
    if (!second) {
      for (k = 0; k < 5; ++k) {
        L[k] = q0[k];
        R[k] = q1[k];
      }
    } else {
      g1 = grad + 15 * (size_t)c1;
      if (!limited) {
        recon3(q0, g0, m->r0 + 3 * f, L);
        recon3(q1, g1, m->r1 + 3 * f, R);
      } else {
        const double dx = m->r0[3 * f] - m->r1[3 * f];
        const double dy = m->r0[3 * f + 1] - m->r1[3 * f + 1];
        const double dz = m->r0[3 * f + 2] - m->r1[3 * f + 2];
        for (k = 0; k < 5; ++k) {
          const double dc = q1[k] - q0[k];
          const double du0 = 2.0 * ((g0[k] * dx + g0[5 + k] * dy) + g0[10 + k] * dz) - dc;
          const double du1 = 2.0 * ((g1[k] * dx + g1[5 + k] * dy) + g1[10 + k] * dz) - dc;
          const double s0 = slope3(p->limiter, du0, dc), s1 = slope3(p->limiter, du1, dc);
          L[k] = q0[k] + 0.5 * s0;
          R[k] = q1[k] - 0.5 * s1;
        }
      }
    }
  } else {
    if (second && !limited) recon3(q0, g0, m->r0 + 3 * f, L);
    else
      for (k = 0; k < 5; ++k) L[k] = q0[k];
    if (kind == 1) {
      for (k = 0; k < 5; ++k) R[k] = p->inlet[k];
    } else if (kind == 4) {
      for (k = 0; k < 5; ++k) R[k] = L[k];
    } else if (p->viscous && second && kind == 2) {
      R[0] = L[0];
      R[1] = -L[1];
      R[2] = -L[2];
      R[3] = -L[3];
      R[4] = L[4];
    } else {
      mirror3(dv, L, R);
    }
  }
  for (d = 0; d < 3; ++d) {
    if (dv[d] >= 0.0) roe3(L, R, d, F + 5 * d);
    else roe3(R, L, d, F + 5 * d);
  }
  if (p->viscous && second && (kind == 0 || kind == 2)) {
    double gu[3], gv[3], gw[3], gT[3];
    prim_grad3(q0, g0, p->cv, gu, gv, gw, gT);
    if (kind == 0) {
      const double eta = m->eta[f], ome = 1.0 - eta;
      double gu1[3], gv1[3], gw1[3], gT1[3], qf[5];
      prim_grad3(q1, g1, p->cv, gu1, gv1, gw1, gT1);
      for (d = 0; d < 3; ++d) {
        gu[d] = eta * gu[d] + ome * gu1[d];
        gv[d] = eta * gv[d] + ome * gv1[d];
        gw[d] = eta * gw[d] + ome * gw1[d];
        gT[d] = eta * gT[d] + ome * gT1[d];
      }
      for (k = 0; k < 5; ++k) qf[k] = eta * q0[k] + ome * q1[k];
      sub_viscous3(qf[1] / qf[0], qf[2] / qf[0], qf[3] / qf[0], gu, gv, gw, gT, p->mu, p->lam,
                   p->kappa, 1, F);
    } else {
      const double *r = m->r0 + 3 * f;
      const double rl = sqrt((r[0] * r[0] + r[1] * r[1]) + r[2] * r[2]);
      const double e[3] = {r[0] / rl, r[1] / rl, r[2] / rl};
      const double u0 = q0[1] / q0[0], v0 = q0[2] / q0[0], w0 = q0[3] / q0[0];
      const double cu = (0.0 - u0) / rl - ((gu[0] * e[0] + gu[1] * e[1]) + gu[2] * e[2]);
      const double cvv = (0.0 - v0) / rl - ((gv[0] * e[0] + gv[1] * e[1]) + gv[2] * e[2]);
      const double cw = (0.0 - w0) / rl - ((gw[0] * e[0] + gw[1] * e[1]) + gw[2] * e[2]);
      for (d = 0; d < 3; ++d) {
        gu[d] = gu[d] + cu * e[d];
        gv[d] = gv[d] + cvv * e[d];
        gw[d] = gw[d] + cw * e[d];
      }
      sub_viscous3(0.0, 0.0, 0.0, gu, gv, gw, gT, p->mu, p->lam, p->kappa, 0, F);
    }
  }
}

void om3_face_flux(const om3_mesh *m, const om3_params *p, const double *q,
                   const double *grad, double *F) {
  int f;
  for (f = 0; f < m->n_faces; ++f) face_flux3(m, p, q, grad, f, F + 15 * (size_t)f);
}

void om3_gather(const om3_mesh *m, const double *F, double *R) {
  int c, k, d, j;
  for (c = 0; c < m->n_cells; ++c) {
    double r[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const double *src = F + 15 * (size_t)m->cell_faces[k];
      for (d = 0; d < 3; ++d) {
        const double s = m->cell_dir[3 * k + d];
        for (j = 0; j < 5; ++j) r[j] += s * src[5 * d + j];
      }
    }
    for (j = 0; j < 5; ++j) R[5 * (size_t)c + j] = r[j];
  }
}

void om3_residual(const om3_mesh *m, const om3_params *p, const double *q, double *R) {
  double *grad = NULL, *F = (double *)malloc(sizeof(double) * 15 * (size_t)(m->n_faces + 1));
  if (p->order == 2) {
    grad = (double *)malloc(sizeof(double) * 15 * (size_t)(m->n_cells + 1));
    om3_gradient(m, q, grad);
  }
  om3_face_flux(m, p, q, grad, F);
  om3_gather(m, F, R);
  free(grad);
  free(F);
}

double om3_dt(const om3_mesh *m, const double *q, double cfl) {
  double best = 1e300;
  int c, k;
  for (c = 0; c < m->n_cells; ++c) {
    const double *qs = q + 5 * (size_t)c;
    const double u = qs[1] / qs[0], v = qs[2] / qs[0], w = qs[3] / qs[0];
    const double snd = sqrt(kGamma * p_of(qs) / qs[0]);
    double lam = 0.0, dtc;
    for (k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const double *dv = m->cell_dir + 3 * k;
      lam += fabs((u * dv[0] + v * dv[1]) + w * dv[2]) +
             snd * sqrt((dv[0] * dv[0] + dv[1] * dv[1]) + dv[2] * dv[2]);
    }
    dtc = cfl * m->cell_vol[c] / (0.5 * lam);
    if (!(dtc > 0)) dtc = 0.0;
    if (dtc < best) best = dtc;
  }
  return best;
}

int om3_rk2(const om3_mesh *m, const om3_params *p, double *q, int nsteps, double cfl,
            double t_end, double *time) {
  const size_t n = 5 * (size_t)m->n_cells;
  double *q0 = (double *)malloc(sizeof(double) * (n + 1));
  double *R = (double *)malloc(sizeof(double) * (n + 1));
  int s, c, j, st;
  if (!q0 || !R) {
    free(q0), free(R);
    return 1;
  }
  for (s = 0; s < nsteps; ++s) {
    double dt = om3_dt(m, q, cfl);
    if (t_end > 0.0 && *time + dt > t_end) dt = t_end - *time;
    if (!(dt > 0.0)) break;
    memcpy(q0, q, sizeof(double) * n);
    for (st = 0; st < 2; ++st) {
      om3_residual(m, p, q, R);
      for (c = 0; c < m->n_cells; ++c) {
        const double f = dt / m->cell_vol[c];
        for (j = 0; j < 5; ++j) {
          const size_t i = 5 * (size_t)c + j;
          if (st == 0) q[i] = q[i] - f * R[i];
          else q[i] = 0.5 * q0[i] + 0.5 * (q[i] - f * R[i]);
        }
      }
    }
    *time += dt;
  }
  free(q0), free(R);
  return 0;
}

void om3_kinetic_energy(const om3_mesh *m, const double *q, double *ke, double *vol) {
  double k = 0.0, v = 0.0;
  int c;
  for (c = 0; c < m->n_cells; ++c) {
    const double *qs = q + 5 * (size_t)c;
    k += 0.5 * ((qs[1] * qs[1] + qs[2] * qs[2]) + qs[3] * qs[3]) / qs[0] * m->cell_vol[c];
    v += m->cell_vol[c];
  }
  *ke = k;
  *vol = v;
}
