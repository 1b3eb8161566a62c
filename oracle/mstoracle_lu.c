/* Oracle restatement of the reference's sparse sweeps (test infrastructure
 * only; see mstoracle.h).
 *
 *   scalar:  lusolver/SparseSolverNUM.cpp  setELE/addELE :115-140,
 *            solveILUSGS :144-212 (X <- (A + L D^-1 U)^-1 (b + L D^-1 U X),
 *            LU_INTERVAL = 5 outer iterations, exit when
 *            1e-20 < max_i |X_i - X_i'| / X_i < 1e-7), solveGS :214-252
 *   block:   lusolver/SparseSolver.cpp  setD/setL/setU :35-48, solveILU
 *            :53-104 with 4x4 blocks (Eigen Matrix4d / Vector4d, the
 *            oracle shim's product order and adjugate inverse), 5 iterations
 *
 * The reference stores each column's L and U entries in insertion order and
 * keeps duplicates; this file applies the same operations in the same order
 * (columns ascending for the forward work, descending for the backward
 * sweep, insertion order inside a column).  Compile with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mstoracle.h"

#define LU_INTERVAL_ 5

typedef struct {
  int n;
  int *ptr, *row;  /* column-wise lists: entries of column c are ptr[c]..ptr[c+1] */
  int *src;        /* insertion index of each entry */
} collist;

/* column lists of the entries with (row > col) for L or (row < col) for U,
 * in insertion order within each column */
static collist make_cols(int dim, int n, const int *rows, const int *cols,
                         int lower) {
  collist cl;
  cl.n = dim;
  cl.ptr = (int *)calloc((size_t)dim + 1, sizeof(int));
  for (int i = 0; i < n; ++i) {
    int keep = lower ? rows[i] > cols[i] : rows[i] < cols[i];
    if (keep) cl.ptr[cols[i] + 1]++;
  }
  for (int c = 0; c < dim; ++c) cl.ptr[c + 1] += cl.ptr[c];
  int tot = cl.ptr[dim];
  cl.row = (int *)calloc((size_t)tot + 1, sizeof(int));
  cl.src = (int *)calloc((size_t)tot + 1, sizeof(int));
  int *fill = (int *)calloc((size_t)dim, sizeof(int));
  for (int i = 0; i < n; ++i) {
    int keep = lower ? rows[i] > cols[i] : rows[i] < cols[i];
    if (!keep) continue;
    int k = cl.ptr[cols[i]] + fill[cols[i]]++;
    cl.row[k] = rows[i];
    cl.src[k] = i;
  }
  free(fill);
  return cl;
}

static void free_cols(collist *cl) {
  free(cl->ptr);
  free(cl->row);
  free(cl->src);
}

int om_lu_scalar(int gs, int dim, int n, const int *rows, const int *cols,
                 const int *ops, const double *vals, const double *b, double *x,
                 int *iterations) {
  double *D = (double *)calloc((size_t)dim, 8);
  /* setELE / addELE: the diagonal is set or accumulated; off-diagonal
   * entries are appended */
  for (int i = 0; i < n; ++i)
    if (rows[i] == cols[i]) {
      if (ops[i] == 1) D[rows[i]] += vals[i];
      else D[rows[i]] = vals[i];
    }
  collist L = make_cols(dim, n, rows, cols, 1), U = make_cols(dim, n, rows, cols, 0);
  double *RHSUx = (double *)calloc((size_t)dim, 8), *RHSLDUx = (double *)calloc((size_t)dim, 8);
  double *RHS = (double *)calloc((size_t)dim, 8), *X1 = (double *)calloc((size_t)dim, 8);
  double *RHS1 = (double *)calloc((size_t)dim, 8);
  int it;
  for (it = 0; it < LU_INTERVAL_; ++it) {
    for (int i = 0; i < dim; ++i) RHSUx[i] = 0., RHSLDUx[i] = 0.;
    for (int c = 0; c < dim; ++c)
      for (int k = U.ptr[c]; k < U.ptr[c + 1]; ++k) RHSUx[U.row[k]] += vals[U.src[k]] * x[c];
    double res = 0;
    if (!gs) {
      for (int i = 0; i < dim; ++i) RHSUx[i] /= D[i];
      for (int c = 0; c < dim; ++c)
        for (int k = L.ptr[c]; k < L.ptr[c + 1]; ++k)
          RHSLDUx[L.row[k]] += vals[L.src[k]] * RHSUx[c];
      for (int i = 0; i < dim; ++i) RHS[i] = b[i] + RHSLDUx[i];
      for (int c = 0; c < dim; ++c)
        for (int k = L.ptr[c]; k < L.ptr[c + 1]; ++k)
          RHS[L.row[k]] -= (vals[L.src[k]]) * (1. / D[c]) * RHS[c];
      for (int i = 0; i < dim; ++i) {
        X1[i] = (1. / D[i]) * RHS[i];
        RHS1[i] = D[i] * X1[i];
      }
      for (int c = dim - 1; c != -1; --c)
        for (int k = U.ptr[c]; k < U.ptr[c + 1]; ++k)
          RHS1[U.row[k]] -= (vals[U.src[k]]) * (1. / D[c]) * RHS1[c];
      for (int i = 0; i < dim; ++i) {
        double r = fabs(x[i] - (1. / D[i]) * RHS1[i]) / x[i];
        if (res < r) res = r;
        x[i] = (1. / D[i]) * RHS1[i];
      }
      if (res > 1e-10 * 1e-10 && res < 1e-7) {
        ++it;
        break;
      }
    } else {
      for (int i = 0; i < dim; ++i) RHS[i] = b[i] - RHSUx[i];
      for (int c = 0; c < dim; ++c)
        for (int k = L.ptr[c]; k < L.ptr[c + 1]; ++k)
          RHS[L.row[k]] -= (vals[L.src[k]]) * (1. / D[c]) * RHS[c];
      for (int i = 0; i < dim; ++i) {
        double r = fabs(x[i] - (1. / D[i]) * RHS[i]) / x[i];
        if (res < r) res = r;
        x[i] = (1. / D[i]) * RHS[i];
      }
      if (res > 1e-10 * 1e-10 && res < 1e-7) {
        ++it;
        break;
      }
    }
  }
  if (iterations) *iterations = it;
  free_cols(&L);
  free_cols(&U);
  free(D), free(RHSUx), free(RHSLDUx), free(RHS), free(X1), free(RHS1);
  return OM_OK;
}

/* ---- 4x4 blocks with the shim's arithmetic (row-major storage) ---- */
static double det3b(double a, double b, double c, double d, double e, double f,
                    double g, double h, double i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}
static void inv4b(const double m[16], double inv[16]) {
  double cof[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      int rr[3], cc[3], t = 0;
      for (int k = 0; k < 4; ++k)
        if (k != i) rr[t++] = k;
      t = 0;
      for (int k = 0; k < 4; ++k)
        if (k != j) cc[t++] = k;
#define M_(r, c) m[4 * rr[r] + cc[c]]
      double v = det3b(M_(0, 0), M_(0, 1), M_(0, 2), M_(1, 0), M_(1, 1), M_(1, 2),
                       M_(2, 0), M_(2, 1), M_(2, 2));
#undef M_
      cof[4 * i + j] = ((i + j) & 1) ? -v : v;
    }
  double det = m[0] * cof[0];
  for (int j = 1; j < 4; ++j) det += m[j] * cof[j];
  double id = 1.0 / det;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) inv[4 * i + j] = cof[4 * j + i] * id;
}
static void mv4(const double a[16], const double x[4], double y[4]) {
  for (int i = 0; i < 4; ++i) {
    double s = a[4 * i] * x[0];
    for (int k = 1; k < 4; ++k) s += a[4 * i + k] * x[k];
    y[i] = s;
  }
}
static void mm4(const double a[16], const double b[16], double c[16]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = a[4 * i] * b[j];
      for (int k = 1; k < 4; ++k) s += a[4 * i + k] * b[4 * k + j];
      c[4 * i + j] = s;
    }
}

int om_lu_block(int dim, int n, const int *rows, const int *cols,
                const double *vals, const double *b, double *x) {
  double *D = (double *)calloc((size_t)16 * dim, 8);
  double *Di = (double *)calloc((size_t)16 * dim, 8);
  for (int i = 0; i < n; ++i)
    if (rows[i] == cols[i]) memcpy(D + 16 * rows[i], vals + 16 * (size_t)i, 128);
  /* D[i].inverse() is recomputed at every use in the reference; it is the
   * same deterministic function of D[i] each time */
  for (int i = 0; i < dim; ++i) inv4b(D + 16 * i, Di + 16 * i);
  collist L = make_cols(dim, n, rows, cols, 1), U = make_cols(dim, n, rows, cols, 0);
  double *RHSUx = (double *)calloc((size_t)4 * dim, 8), *RHSLDUx = (double *)calloc((size_t)4 * dim, 8);
  double *RHS = (double *)calloc((size_t)4 * dim, 8), *X1 = (double *)calloc((size_t)4 * dim, 8);
  double *RHS1 = (double *)calloc((size_t)4 * dim, 8);
  double t[4], M[16];
  for (int it = 0; it < LU_INTERVAL_; ++it) {
    memset(RHSUx, 0, sizeof(double) * 4 * dim);
    memset(RHSLDUx, 0, sizeof(double) * 4 * dim);
    for (int c = 0; c < dim; ++c)
      for (int k = U.ptr[c]; k < U.ptr[c + 1]; ++k) {
        mv4(vals + 16 * (size_t)U.src[k], x + 4 * c, t);
        for (int j = 0; j < 4; ++j) RHSUx[4 * U.row[k] + j] += t[j];
      }
    for (int i = 0; i < dim; ++i) {
      mv4(Di + 16 * i, RHSUx + 4 * i, t);
      memcpy(RHSUx + 4 * i, t, 32);
    }
    for (int c = 0; c < dim; ++c)
      for (int k = L.ptr[c]; k < L.ptr[c + 1]; ++k) {
        mv4(vals + 16 * (size_t)L.src[k], RHSUx + 4 * c, t);
        for (int j = 0; j < 4; ++j) RHSLDUx[4 * L.row[k] + j] += t[j];
      }
    for (int i = 0; i < 4 * dim; ++i) RHS[i] = b[i] + RHSLDUx[i];
    for (int c = 0; c < dim; ++c)
      for (int k = L.ptr[c]; k < L.ptr[c + 1]; ++k) {
        mm4(vals + 16 * (size_t)L.src[k], Di + 16 * c, M);
        mv4(M, RHS + 4 * c, t);
        for (int j = 0; j < 4; ++j) RHS[4 * L.row[k] + j] -= t[j];
      }
    for (int i = 0; i < dim; ++i) {
      mv4(Di + 16 * i, RHS + 4 * i, X1 + 4 * i);
      mv4(D + 16 * i, X1 + 4 * i, RHS1 + 4 * i);
    }
    for (int c = dim - 1; c != -1; --c)
      for (int k = U.ptr[c]; k < U.ptr[c + 1]; ++k) {
        mm4(vals + 16 * (size_t)U.src[k], Di + 16 * c, M);
        mv4(M, RHS1 + 4 * c, t);
        for (int j = 0; j < 4; ++j) RHS1[4 * U.row[k] + j] -= t[j];
      }
    for (int i = 0; i < dim; ++i) mv4(Di + 16 * i, RHS1 + 4 * i, x + 4 * i);
  }
  free_cols(&L);
  free_cols(&U);
  free(D), free(Di), free(RHSUx), free(RHSLDUx), free(RHS), free(X1), free(RHS1);
  return OM_OK;
}
