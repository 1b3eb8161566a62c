/* Oracle restatement of the reference's pressure-based SIMPLE solver
 * (pSolver/SolverSIMPLE.cpp, the PSOLVER the reference's CONST.h selects).
 *
 * TEST INFRASTRUCTURE ONLY (see mstoracle.h): the checker of the CUDA
 * SIMPLE path and the CPU baseline of the bench, never a product path.
 *
 * Parity pinning: checked bit-for-bit against the reference's own
 * SolverSIMPLE compiled from its sources (oracle/ref/harness_simple.cpp,
 * one OpenMP thread) on the shipped meshes (tests/test_simple.py), with
 * the Eigen arithmetic of the project's shim (oracle/ref/eigen_shim).
 *
 * One SIMPLE iteration of SolverSIMPLE::solve (:48-80) as the reference
 * runs it:
 *   updateFacePUVT   face (p,u,v,T) by zone type (:82-193)
 *   updateUStar      u momentum system, Gauss-Seidel (:247-344)
 *   updateVStar      v momentum system, Gauss-Seidel (:346-439)
 *   updateFacePUVT   again, with the new u and v
 *   updatePUV2       pressure-correction system, Gauss-Seidel,
 *                    p += SIMPLE_ALPHA_P p' (:712-838)
 *   updateT          explicit energy update (:1315-1346)
 *   residual         max |new - old_n| / (old_n + EOR), old = new (:62-71)
 * updateGrad and updateFacePUVTRhieChow also run in the reference, but what
 * they write (cell and face gradients, the Rhie-Chow face values, the
 * first-order upwind face values and flags) is read nowhere on this path:
 * every quantity above reads the central face values only.  They are not
 * restated.
 *
 * Compile with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mstoracle.h"

#define CP_ 1002.12
#define CV_ 715.8
#define EOR_ 1e-10

/* getPBasedRho (work/FUNCTION.cpp:25-27): p / (CP-CV) / T */
static double rho_pb(const double *x) { return x[0] / (CP_ - CV_) / x[3]; }

/* getP / getT (work/FUNCTION.cpp:7-14) */
static double q_p(const double q[4]) {
  return (q[3] - 0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0]) * (1.4 - 1);
}
static double q_t(const double q[4]) {
  return (q[3] - 0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0]) / q[0] / CV_;
}

void om_q_to_puvt(int n, const double *q, double *puvt) {
  /* Time::initialization (time/Time.cpp:21-23) */
  for (int i = 0; i < n; ++i) {
    const double *a = q + 4 * (size_t)i;
    double *o = puvt + 4 * (size_t)i;
    o[0] = q_p(a);
    o[1] = a[1] / a[0];
    o[2] = a[2] / a[0];
    o[3] = q_t(a);
  }
}

void om_simple_default_params(om_simple_params *p) {
  /* CONST.h: STEP_TIME 4e+3, SIMPLE_INTERVAL 5, SIMPLE_ALPHA_P 0.3,
   * FLAG_WALLSMOOTH 1; inlet (SolverSIMPLE.cpp:110-112) = (getP(inletQ),
   * inletu, inletv, inletT) and outlet pressure (:168-175) = getP(iniQ),
   * both from the reference's initial state */
  double q[4];
  om_reference_inlet(q);
  p->dt = 1. / 4e+3;
  p->alpha_p = 0.3;
  p->n_inner = 5;
  p->wall_smooth = 1;
  p->inlet[0] = q_p(q);
  p->inlet[1] = 0;
  p->inlet[2] = 0;
  p->inlet[3] = 1 / 286.32;
  p->p_out = q_p(q);
}

/* updateFacePUVT (:82-193): central face values of the handled zone types;
 * faces of other types keep what they hold */
static void face_pass(const om_mesh *m, const om_simple_params *p,
                      const double *puvt, double *fc) {
  for (int z = 0; z < m->n_zones; ++z) {
    const int type = m->zone[4 * z + 3];
    const int a = m->zone[4 * z + 1] - 1, b = m->zone[4 * z + 2];
    for (int f = a; f < b; ++f) {
      double *o = fc + 4 * (size_t)f;
      const double *in = puvt + 4 * (size_t)m->face_cells[2 * f];
      if (type == 2) {
        const double *c1 = puvt + 4 * (size_t)m->face_cells[2 * f + 1];
        const double e = m->face_eta0[f];
        for (int k = 0; k < 4; ++k) o[k] = in[k] * e + (1 - e) * c1[k];
      } else if (type == 10) {
        for (int k = 0; k < 4; ++k) o[k] = p->inlet[k];
      } else if (type == 3) {
        const int n0 = m->face_nodes[2 * f], n1 = m->face_nodes[2 * f + 1];
        const double dX = m->node_xy[2 * n1] - m->node_xy[2 * n0];
        const double dY = m->node_xy[2 * n1 + 1] - m->node_xy[2 * n0 + 1];
        double out[4] = {in[0], in[1], in[2], in[3]};
        if (p->wall_smooth) {
          out[2] = (2 * dX * dY * in[1] - (dX * dX - dY * dY) * in[2]) / (dX * dX + dY * dY);
          out[1] = (2 * dX * dY * in[2] - (dY * dY - dX * dX) * in[1]) / (dX * dX + dY * dY);
        } else {
          out[2] = 0;
          out[1] = 0;
        }
        for (int k = 0; k < 4; ++k) o[k] = (out[k] + in[k]) / 2.0;
      } else if (type == 5) {
        for (int k = 0; k < 4; ++k) o[k] = in[k];
        o[0] = p->p_out;
      }
    }
  }
}

typedef struct {
  int n, cap;
  int *rows, *cols, *ops;
  double *vals;
} ins_list;

static void ins(ins_list *l, int r, int c, int op, double v) {
  if (l->n == l->cap) {
    l->cap = l->cap ? 2 * l->cap : 1024;
    l->rows = (int *)realloc(l->rows, (size_t)l->cap * sizeof(int));
    l->cols = (int *)realloc(l->cols, (size_t)l->cap * sizeof(int));
    l->ops = (int *)realloc(l->ops, (size_t)l->cap * sizeof(int));
    l->vals = (double *)realloc(l->vals, (size_t)l->cap * sizeof(double));
  }
  l->rows[l->n] = r, l->cols[l->n] = c, l->ops[l->n] = op, l->vals[l->n] = v;
  ++l->n;
}

/* the cell classes in the reference's assembly order: inner, bond2, bond1 */
static void class_list(const om_mesh *m, int k, const int **list, int *n) {
  if (k == 0) *list = m->inner, *n = m->n_inner;
  else if (k == 1) *list = m->bond2, *n = m->n_bond2;
  else *list = m->bond1, *n = m->n_bond1;
}

/* updateUStar / updateVStar (:247-439).  Both systems have the same matrix
 * (the density uses p and T only, which neither solve changes); the right
 * sides differ. */
static void momentum(const om_mesh *m, const om_simple_params *p, const double *puvt,
                     const double *oldn, const double *fc, ins_list *L, double *bu,
                     double *bv, double *uD) {
  const double dt = p->dt;
  L->n = 0;
  for (int k = 0; k < 3; ++k) {
    const int *list;
    int n;
    class_list(m, k, &list, &n);
    for (int i = 0; i < n; ++i) {
      const int c = list[i];
      const double V = m->cell_vol[c];
      double cofC = rho_pb(puvt + 4 * c) * V / dt;
      const double ro = rho_pb(oldn + 4 * c);
      const double rtu = (k == 0) ? ro * oldn[4 * c + 1] * V / dt : ro * V * oldn[4 * c + 1] / dt;
      const double rtv = ro * V * oldn[4 * c + 2] / dt;
      double rpu = 0, rpv = 0, rbu = 0, rbv = 0;
      for (int j = m->cell_ptr[c]; j < m->cell_ptr[c + 1]; ++j) {
        const int f = m->cell_faces[j];
        const double *x = fc + 4 * (size_t)f;
        const double d0 = m->cell_dof[2 * j], d1 = m->cell_dof[2 * j + 1];
        const double rf = rho_pb(x);
        if (k != 2 || f < m->n_int_faces) {
          const double e = m->cell_eta0c[j];
          double t = (rf * x[1]) * d0;
          t += (rf * x[2]) * d1;
          cofC += t * e;
          ins(L, c, m->cell_nb[j], 1, t * (1 - e));
        } else {
          const double su = -rf * x[1], sv = -rf * x[2];
          double tu = (su * x[1]) * d0;
          tu += (su * x[2]) * d1;
          double tv = (sv * x[1]) * d0;
          tv += (sv * x[2]) * d1;
          rbu += tu;
          rbv += tv;
        }
        rpu += -x[0] * d0;
        rpv += -x[0] * d1;
      }
      ins(L, c, c, 0, cofC);
      uD[c] = cofC;
      bu[c] = (k == 2) ? rpu + rtu + rbu : rpu + rtu;
      bv[c] = (k == 2) ? rpv + rtv + rbv : rpv + rtv;
    }
  }
}

/* updatePUV2 (:712-838): pressure-correction system */
static void pressure(const om_mesh *m, const om_simple_params *p, const double *puvt,
                     const double *oldn, const double *fc, const double *uD, ins_list *L,
                     double *b) {
  const double dt = p->dt;
  L->n = 0;
  for (int k = 0; k < 3; ++k) {
    const int *list;
    int n;
    class_list(m, k, &list, &n);
    for (int i = 0; i < n; ++i) {
      const int c = list[i];
      const double V = m->cell_vol[c];
      const double pc = puvt[4 * c];
      double cofPC = V / dt / (CP_ - CV_) / puvt[4 * c + 3];
      double rhs = -V * (rho_pb(puvt + 4 * c) - rho_pb(oldn + 4 * c)) / dt;
      for (int j = m->cell_ptr[c]; j < m->cell_ptr[c + 1]; ++j) {
        const int f = m->cell_faces[j];
        const double *x = fc + 4 * (size_t)f;
        const double d0 = m->cell_dof[2 * j], d1 = m->cell_dof[2 * j + 1];
        const double rf = rho_pb(x);
        const double dot = x[1] * d0 + x[2] * d1;
        rhs += -rf * dot;
        if (k == 2 && m->face_type[f] != 2) continue;
        const double e = m->cell_eta0c[j];
        const int F = m->cell_nb[j];
        const double rx = m->cell_ctr[2 * c] - m->cell_ctr[2 * F];
        const double ry = m->cell_ctr[2 * c + 1] - m->cell_ctr[2 * F + 1];
        double s = rx * rx;
        s += ry * ry;
        const double dist = sqrt(s);
        double sd = d0 * d0;
        sd += d1 * d1;
        const double dn = sqrt(sd);
        /* both coefficients divide by the u diagonal of the neighbour
         * (:733-734): the u and v diagonals are equal here */
        const double cu = (e * V / uD[c] + (1 - e) * m->cell_vol[F] / uD[F]) / dist * d0 / dn;
        const double cv = (e * V / uD[c] + (1 - e) * m->cell_vol[F] / uD[F]) / dist * d1 / dn;
        cofPC += e * rf / pc * dot;
        double cofPF = (1 - e) * rf / pc * dot;
        cofPC += rf * (cu * d0 + cv * d1);
        cofPF += -rf * (cu * d0 + cv * d1);
        ins(L, c, F, 1, cofPF);
      }
      ins(L, c, c, k == 2 ? 0 : 1, cofPC);
      b[c] = rhs;
    }
  }
}

/* updateT (:1315-1346), FLAG_PBASED_EXPLICIT 1 */
static void energy(const om_mesh *m, const om_simple_params *p, double *puvt,
                   const double *oldn, const double *fc) {
  for (int c = 0; c < m->n_cells; ++c) {
    double rhs = 0;
    for (int j = m->cell_ptr[c]; j < m->cell_ptr[c + 1]; ++j) {
      const int f = m->cell_faces[j];
      const double *x = fc + 4 * (size_t)f;
      const double d0 = m->cell_dof[2 * j], d1 = m->cell_dof[2 * j + 1];
      rhs += -rho_pb(x) * x[3] * (d0 * x[1] + d1 * x[2]);
      rhs += 1 / CP_ * x[0] * (d0 + d1);
    }
    double *o = puvt + 4 * (size_t)c;
    const double *a = oldn + 4 * (size_t)c;
    o[3] = (rhs / m->cell_vol[c] * p->dt + 1 / CP_ * (o[0] - a[0]) + rho_pb(a) * a[3]) /
           rho_pb(o);
  }
}

/* max over cells of |new - old| / (old + eps), NaN and negative quotients
 * never replacing the running value (SolverSIMPLE.cpp:64-69, Time.cpp:66-72) */
static void rel_change(int n, const double *nw, const double *od, int eps, double r[4]) {
  for (int k = 0; k < 4; ++k) r[k] = 0;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 4; ++k) {
      const double o = od[4 * i + k];
      const double q = fabs(nw[4 * i + k] - o) / (eps ? o + EOR_ : o);
      if (r[k] < q) r[k] = q;
    }
}

int om_simple_step(const om_mesh *m, const om_simple_params *p, double *puvt,
                   double *fc, int nsteps, double *time_rows, double *inner_rows,
                   int *gs_iters) {
  const int nC = m->n_cells;
  double *oldn = (double *)malloc((size_t)nC * 4 * sizeof(double));
  double *bu = (double *)malloc((size_t)nC * sizeof(double));
  double *bv = (double *)malloc((size_t)nC * sizeof(double));
  double *uD = (double *)malloc((size_t)nC * sizeof(double));
  double *x = (double *)malloc((size_t)nC * sizeof(double));
  ins_list L = {0, 0, NULL, NULL, NULL, NULL};
  for (int s = 0; s < nsteps; ++s) {
    /* SolverSIMPLE's constructor: old time level = old = new (:34-36) */
    memcpy(oldn, puvt, (size_t)nC * 4 * sizeof(double));
    for (int it = 0; it < p->n_inner; ++it) {
      int its[3];
      face_pass(m, p, puvt, fc);
      momentum(m, p, puvt, oldn, fc, &L, bu, bv, uD);
      for (int c = 0; c < nC; ++c) x[c] = puvt[4 * c + 1];
      om_lu_scalar(1, nC, L.n, L.rows, L.cols, L.ops, L.vals, bu, x, &its[0]);
      for (int c = 0; c < nC; ++c) puvt[4 * c + 1] = x[c], x[c] = puvt[4 * c + 2];
      om_lu_scalar(1, nC, L.n, L.rows, L.cols, L.ops, L.vals, bv, x, &its[1]);
      for (int c = 0; c < nC; ++c) puvt[4 * c + 2] = x[c];
      face_pass(m, p, puvt, fc);
      pressure(m, p, puvt, oldn, fc, uD, &L, bu);
      for (int c = 0; c < nC; ++c) x[c] = 0;
      om_lu_scalar(1, nC, L.n, L.rows, L.cols, L.ops, L.vals, bu, x, &its[2]);
      for (int c = 0; c < nC; ++c) puvt[4 * c] += p->alpha_p * x[c];
      energy(m, p, puvt, oldn, fc);
      if (inner_rows)
        rel_change(nC, puvt, oldn, 1, inner_rows + 4 * ((size_t)s * p->n_inner + it));
      if (gs_iters)
        for (int k = 0; k < 3; ++k) gs_iters[3 * ((size_t)s * p->n_inner + it) + k] = its[k];
    }
    if (time_rows) rel_change(nC, puvt, oldn, 0, time_rows + 4 * (size_t)s);
  }
  free(L.rows), free(L.cols), free(L.ops), free(L.vals);
  free(oldn), free(bu), free(bv), free(uD), free(x);
  return OM_OK;
}
