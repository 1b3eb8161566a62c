/* CPU restatement of MST-CFD's result writer and text checkpoint.
 *
 * TEST INFRASTRUCTURE ONLY (see mstoracle.h): the checker of the product's
 * mst_node_values / mst_write_plt / mst_write_cell_text.
 *
 * Parity pinning: om_write_plt restates Work::writedataRhoBasedMshNodePlt
 * (work/Work.cpp:204-319) and is compared byte-for-byte with the file the
 * reference's own member function writes (oracle/ref/harness_io.cpp) in
 * tests/test_io.py.  Compiled with -ffp-contract=off like the rest of the
 * oracle, so every operation rounds in the reference's order.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mstoracle.h"
#include "mstoracle_io.h"

/* Work.cpp:244-283 face values, then :287-295 node averages.  quirks: the
 * weight of every face of node i is 1/area of face i (the reference indexes
 * the face list by the node id); else the face's own 1/area.  Face types
 * other than 2/10/3/5 are left unset by the reference; here they take the
 * cell value (callers comparing with the reference avoid them). */
int om_node_values(const om_mesh *m, const double *q, int quirks, double cv,
                   double *node_q, double *node_vars) {
  const int nN = m->n_nodes, nF = m->n_faces;
  if (quirks && nN > nF) return OM_EINVAL;
  double *fq = (double *)malloc(sizeof(double) * 4 * (size_t)(nF > 0 ? nF : 1));
  int *cnt = (int *)calloc((size_t)nN + 1, sizeof(int));
  int *lst;
  int f, i, k, j;
  for (f = 0; f < nF; ++f) {
    const double *q0 = q + 4 * (size_t)m->face_cells[2 * f];
    if (m->face_type[f] == 2) {
      const double e = m->face_eta0[f];
      const double *q1 = q + 4 * (size_t)m->face_cells[2 * f + 1];
      for (j = 0; j < 4; ++j) {
        double v = e * q0[j];
        v += (1 - e) * q1[j];
        fq[4 * (size_t)f + j] = v;
      }
    } else {
      for (j = 0; j < 4; ++j) fq[4 * (size_t)f + j] = q0[j];
    }
  }
  /* Node::pNbFaces in reader order (MshBlock.cpp:231-232): faces ascending */
  for (f = 0; f < nF; ++f)
    for (k = 0; k < 2; ++k) cnt[m->face_nodes[2 * f + k] + 1]++;
  for (i = 0; i < nN; ++i) cnt[i + 1] += cnt[i];
  lst = (int *)malloc(sizeof(int) * (size_t)(cnt[nN] > 0 ? cnt[nN] : 1));
  {
    int *fill = (int *)malloc(sizeof(int) * (size_t)(nN > 0 ? nN : 1));
    memcpy(fill, cnt, sizeof(int) * (size_t)nN);
    for (f = 0; f < nF; ++f)
      for (k = 0; k < 2; ++k) lst[fill[m->face_nodes[2 * f + k]]++] = f;
    free(fill);
  }
  for (i = 0; i < nN; ++i) {
    double acc[4] = {0, 0, 0, 0}, d = 0;
    for (k = cnt[i]; k < cnt[i + 1]; ++k) {
      const int g = lst[k];
      const double w = quirks ? 1 / m->face_area[i] : 1 / m->face_area[g];
      for (j = 0; j < 4; ++j) acc[j] += w * fq[4 * (size_t)g + j];
      d += w;
    }
    for (j = 0; j < 4; ++j) acc[j] /= d;
    if (node_q)
      for (j = 0; j < 4; ++j) node_q[4 * (size_t)i + j] = acc[j];
    if (node_vars) {
      /* work/FUNCTION.cpp:8-20 */
      const double gm = 1.4;
      double *o = node_vars + 6 * (size_t)i;
      const double T = (acc[3] - 0.5 * (acc[1] * acc[1] + acc[2] * acc[2]) / acc[0]) / acc[0] / cv;
      const double p = (acc[3] - 0.5 * (acc[1] * acc[1] + acc[2] * acc[2]) / acc[0]) * (gm - 1);
      const double ma = sqrt((acc[1] * acc[1] + acc[2] * acc[2]) / (gm * p * acc[0]));
      o[0] = acc[0];
      o[1] = acc[1] / acc[0];
      o[2] = acc[2] / acc[0];
      o[3] = T;
      o[4] = p;
      o[5] = ma;
    }
  }
  free(lst);
  free(cnt);
  free(fq);
  return OM_OK;
}

/* Cell node lists (MshBlock.cpp:335-367): faces of the cell in order, each
 * node appended once; a 4-node cell swaps nodes 2 and 3 when
 * (n0 - n1).(n2 - n3) < 0.  ptr [n_cells+1], ids [4 n_cells] max. */
void om_cell_nodes(const om_mesh *m, int *ptr, int *ids) {
  int c, k, j, t = 0;
  ptr[0] = 0;
  for (c = 0; c < m->n_cells; ++c) {
    const int b = t;
    for (k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const int f = m->cell_faces[k];
      for (j = 0; j < 2; ++j) {
        const int n = m->face_nodes[2 * f + j];
        int have = 0, i;
        for (i = b; i < t; ++i) have |= ids[i] == n;
        if (!have) ids[t++] = n;
      }
    }
    if (t - b == 4) {
      const double *p0 = m->node_xy + 2 * (size_t)ids[b], *p1 = m->node_xy + 2 * (size_t)ids[b + 1];
      const double *p2 = m->node_xy + 2 * (size_t)ids[b + 2], *p3 = m->node_xy + 2 * (size_t)ids[b + 3];
      double dot = (p0[0] - p1[0]) * (p2[0] - p3[0]);
      dot += (p0[1] - p1[1]) * (p2[1] - p3[1]);
      if (dot < 0) {
        const int s = ids[b + 2];
        ids[b + 2] = ids[b + 3];
        ids[b + 3] = s;
      }
    }
    ptr[c + 1] = t;
  }
}

/* The reference-mode file of Work::writedataRhoBasedMshNodePlt. */
int om_write_plt(const om_mesh *m, const double *q, double cv, int zone_t,
                 const char *path) {
  const int nN = m->n_nodes, nC = m->n_cells;
  double *v = (double *)malloc(sizeof(double) * 6 * (size_t)(nN > 0 ? nN : 1));
  int *ptr = (int *)malloc(sizeof(int) * ((size_t)nC + 1));
  int *ids = (int *)malloc(sizeof(int) * 4 * (size_t)(nC > 0 ? nC : 1) + 64);
  FILE *f;
  int i, k, st = om_node_values(m, q, 1, cv, NULL, v);
  if (st != OM_OK) {
    free(v); free(ptr); free(ids);
    return st;
  }
  om_cell_nodes(m, ptr, ids);
  f = fopen(path, "wb");
  if (!f) {
    free(v); free(ptr); free(ids);
    return OM_EINVAL;
  }
  fprintf(f, "\"TITLE = \"Example: Variable and Connectivity List Sharing\"\n");
  fprintf(f, "VARIABLES = \"X\", \"Y\", \"rho\" , \"u\" , \"v\" , \"T\" , \"p\" , \"Ma\" \n");
  fprintf(f, "ZONE T=\"%d\", DATAPACKING=POINT, NODES=%d, ELEMENTS=%d, ZONETYPE=FEQUADRILATERAL\n",
          zone_t, nN, nC);
  for (i = 0; i < nN; ++i) {
    fprintf(f, "%.15f %.15f ", m->node_xy[2 * (size_t)i], m->node_xy[2 * (size_t)i + 1]);
    for (k = 0; k < 6; ++k) fprintf(f, "%.15f ", v[6 * (size_t)i + k]);
    fprintf(f, "\n");
  }
  for (i = 0; i < nC; ++i) {
    for (k = ptr[i]; k < ptr[i + 1]; ++k) fprintf(f, "%d ", ids[k] + 1);
    fprintf(f, "\n");
  }
  fclose(f);
  free(v); free(ptr); free(ids);
  return OM_OK;
}

/* Work::writedataCellContinue (Work.cpp:483-514): 4 numbers per cell. */
int om_write_cell_text(int n_cells, const double *q, const char *path) {
  FILE *f = fopen(path, "wb");
  int i, k;
  if (!f) return OM_EINVAL;
  for (i = 0; i < n_cells; ++i) {
    for (k = 0; k < 4; ++k) fprintf(f, "%.15f ", q[4 * (size_t)i + k]);
    fprintf(f, "\n");
  }
  fclose(f);
  return OM_OK;
}
