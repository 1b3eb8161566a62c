/* CPU restatement of MST-CFD's density-based residual path (oracle; test
 * infrastructure only -- see mstoracle.h).  Compile with
 * -ffp-contract=off: every product and sum below is rounded separately, in
 * the order the reference (with the oracle's Eigen-subset shim) evaluates
 * it, so results are bit-identical to oracle/_ref on x86-64 and aarch64. */
#include "mstoracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define GAMMA_ 1.4
#define EOR_ 1e-10
#define EOR2_ 1e-7

/* ------------------------------------------------------------------ */
/* thermo helpers, work/FUNCTION.cpp:3-15 (2D momentum only)           */
/* ------------------------------------------------------------------ */
static double th_p(const double q[4]) {
  double ke = 0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0];
  return (q[3] - ke) * (GAMMA_ - 1);
}
static double th_ht(const double q[4]) {
  double p = th_p(q);
  return (q[3] + p) / q[0];
}

void om_reference_inlet(double q[4]) {
  /* CONST.h:70-83: rho = 1, u = v = 0, E = rho*(T*CV + 0.5*|u|^2) with
   * T = 1/286.32 and CV = 715.8 (macro expansion evaluates 1/286.32*715.8
   * left to right). */
  double T = 1 / 286.32;
  q[0] = 1;
  q[1] = 1.0 * 0;
  q[2] = 1.0 * 0;
  q[3] = 1 * (T * 715.8 + 0.5 * (0 * 0 + 0 * 0));
}

void om_default_params(om_params *p) {
  p->flux = OM_AUSM;
  p->order = 1;
  om_reference_inlet(p->inlet_q);
}

/* ------------------------------------------------------------------ */
/* AUSM+ : rhoSolver/SolverAusm.cpp:3-26 (set), :53-63 (solverAll),    */
/* :105-143 (calculateMachAndPFace_AusmPlus)                           */
/* ------------------------------------------------------------------ */
void om_ausm_flux(const double ql[4], const double qr[4], int d,
                  double f[4]) {
  /* set(): interface speed from the critical speeds a* */
  double aLs = sqrt(2 * th_ht(ql) * (GAMMA_ - 1) / (GAMMA_ + 1));
  double aRs = sqrt(2 * th_ht(qr) * (GAMMA_ - 1) / (GAMMA_ + 1));
  double UL = sqrt((ql[1] * ql[1] + ql[2] * ql[2]) / ql[0] / ql[0]);
  double UR = sqrt((qr[1] * qr[1] + qr[2] * qr[2]) / qr[0] / qr[0]);
  double aL = aLs * aLs / (aLs < UL ? UL : aLs);   /* std::max */
  double aR = aRs * aRs / (aRs < UR ? UR : aRs);
  double aF = (aR < aL) ? aR : aL;                 /* std::min */
  double pL = th_p(ql), pR = th_p(qr);
  /* solverAll(d) */
  double mL = ql[d + 1] / ql[0] / aF;
  double mR = qr[d + 1] / qr[0] / aF;
  /* calculateMachAndPFace_AusmPlus: flux weights use the true sound speeds */
  double fL[4] = {ql[0], ql[1], ql[2], ql[3] + th_p(ql)};
  double fR[4] = {qr[0], qr[1], qr[2], qr[3] + th_p(qr)};
  aL = sqrt(GAMMA_ * th_p(ql) / ql[0]);
  aR = sqrt(GAMMA_ * th_p(qr) / qr[0]);
  double mp, mm, pp, pm;
  /* abs(mach <= 1) in the reference is the test mach <= 1 */
  if (mL <= 1)
    mp = 0.25 * (mL + 1) * (mL + 1) + 0.125 * (mL * mL - 1) * (mL * mL - 1);
  else
    mp = 0.5 * (mL + fabs(mL));
  if (mR <= 1)
    mm = -0.25 * (mR - 1) * (mR - 1) - 0.125 * (mR * mR - 1) * (mR * mR - 1);
  else
    mm = 0.5 * (mR - fabs(mR));
  if (mL <= 1)
    pp = pL * 0.25 * (mL + 1) * (mL + 1) * (2 - mL) +
         0.1875 * mL * (mL * mL - 1) * (mL * mL - 1);
  else
    pp = pL * 0.5 * (mL + fabs(mL)) / mL;
  if (mR <= 1)
    pm = pR * 0.25 * (mR - 1) * (mR - 1) * (2 + mR) -
         0.1875 * mR * (mR * mR - 1) * (mR * mR - 1);
  else
    pm = pR * 0.5 * (mR - fabs(mR)) / mR;
  double mF = mm + mp;
  double pF = pm + pp;
  for (int k = 0; k < 4; ++k) {
    double a = mF * (aL * fL[k] + aR * fR[k]);
    double b = fabs(mF) * (aR * fR[k] - aL * fL[k]);
    f[k] = 0.5 * (a - b);
  }
  f[d + 1] += pF;
}

/* ------------------------------------------------------------------ */
/* Roe : rhoSolver/SolverRoe.cpp:3-16 (set), :70-111 (solverAll),      */
/* :114-123 (entropyRefine).  |A| = R |Lambda| R^-1 with R^-1 from the */
/* adjugate formula of the oracle's Eigen shim.                        */
/* ------------------------------------------------------------------ */
static double entropy_fix(double x) {
  double e = 0.125;
  if (x > e) return x;
  return (x * x + e * e) / 2 / e;
}
static double det3(double a, double b, double c, double d, double e, double f,
                   double g, double h, double i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}
/* m, inv: row-major 4x4 */
static void inv4(const double m[16], double inv[16]) {
  double cof[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      int rr[3], cc[3], n;
      n = 0;
      for (int k = 0; k < 4; ++k)
        if (k != i) rr[n++] = k;
      n = 0;
      for (int k = 0; k < 4; ++k)
        if (k != j) cc[n++] = k;
#define M_(r, c) m[4 * rr[r] + cc[c]]
      double v = det3(M_(0, 0), M_(0, 1), M_(0, 2), M_(1, 0), M_(1, 1),
                      M_(1, 2), M_(2, 0), M_(2, 1), M_(2, 2));
#undef M_
      cof[4 * i + j] = ((i + j) & 1) ? -v : v;
    }
  double det = m[0] * cof[0];
  for (int j = 1; j < 4; ++j) det += m[j] * cof[j];
  double id = 1.0 / det;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) inv[4 * i + j] = cof[4 * j + i] * id;
}
static void mat4_mul(const double a[16], const double b[16], double c[16]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = a[4 * i] * b[j];
      for (int k = 1; k < 4; ++k) s += a[4 * i + k] * b[4 * k + j];
      c[4 * i + j] = s;
    }
}

void om_roe_flux(const double ql[4], const double qr[4], int d, double f[4]) {
  double D = sqrt(fabs(qr[0] / ql[0]));
  double u[2];
  for (int k = 0; k < 2; ++k)
    u[k] = (ql[k + 1] / ql[0] + D * qr[k + 1] / qr[0]) / (1. + D);
  double H = (th_ht(ql) + D * th_ht(qr)) / (1. + D);
  double un = sqrt(u[0] * u[0] + u[1] * u[1]);
  double a = sqrt(fabs((GAMMA_ - 1.) * (H - 0.5 * (un * un))));
  double lam[16] = {0};
  double ud = u[d];
  lam[0] = entropy_fix(fabs(ud - a));
  lam[5] = entropy_fix(fabs(ud));
  lam[10] = entropy_fix(fabs(ud));
  lam[15] = entropy_fix(fabs(ud + a));
  double R[16], FL[4], FR[4];
  double ke = 0.5 * (u[0] * u[0] + u[1] * u[1]);
  if (d == 0) {
    double r[16] = {1, 1, 0, 1,
                    u[0] - a, u[0], 0, u[0] + a,
                    u[1], u[1], 1, u[1],
                    H - u[0] * a, ke, u[1], H + u[0] * a};
    memcpy(R, r, sizeof r);
    FL[0] = ql[1];
    FL[1] = ql[1] * ql[1] / (ql[0] + EOR_) + th_p(ql);
    FL[2] = ql[1] * ql[2] / (ql[0] + EOR_);
    FL[3] = th_ht(ql) * ql[1];
    FR[0] = qr[1];
    FR[1] = qr[1] * qr[1] / (qr[0] + EOR_) + th_p(qr);
    FR[2] = qr[1] * qr[2] / (qr[0] + EOR_);
    FR[3] = th_ht(qr) * qr[1];
  } else {
    double r[16] = {1, 1, 0, 1,
                    u[0], u[0], 1, u[0],
                    u[1] - a, u[1], 0, u[1] + a,
                    H - u[1] * a, ke, u[0], H + u[1] * a};
    memcpy(R, r, sizeof r);
    FL[0] = ql[2];
    FL[1] = ql[1] * ql[2] / (ql[0] + EOR_);
    FL[2] = ql[2] * ql[2] / (ql[0] + EOR_) + th_p(ql);
    FL[3] = th_ht(ql) * ql[2];
    FR[0] = qr[2];
    FR[1] = qr[1] * qr[2] / (qr[0] + EOR_);
    FR[2] = qr[2] * qr[2] / (qr[0] + EOR_) + th_p(qr);
    FR[3] = th_ht(qr) * qr[2];
  }
  double Ri[16], RL[16], A[16];
  inv4(R, Ri);
  mat4_mul(R, lam, RL);
  mat4_mul(RL, Ri, A);
  double dU[4];
  for (int k = 0; k < 4; ++k) dU[k] = qr[k] - ql[k];
  for (int k = 0; k < 4; ++k) {
    double s = (0.5 * A[4 * k]) * dU[0];
    for (int j = 1; j < 4; ++j) s += (0.5 * A[4 * k + j]) * dU[j];
    f[k] = 0.5 * (FL[k] + FR[k]) - s;
  }
}

typedef void (*flux_fn)(const double *, const double *, int, double *);

/* ------------------------------------------------------------------ */
/* mesh reader: MshBlock::splitInformationData2D / dataToMesh2D        */
/* (mesh/MshBlock.cpp:75-432), FUNCTION.cpp:41-72 (hex/brackets)       */
/* ------------------------------------------------------------------ */
/* hexStringToInt: lower-case hex digits; any other character still takes
 * a digit position but adds nothing. */
static int hex_token(const char *s, size_t n) {
  int v = 0;
  for (size_t i = 0; i < n; ++i) {
    int w = 0;
    char c = s[i];
    if (c >= 'a' && c <= 'f') w = c - 'a' + 10;
    else if (c >= '0' && c <= '9') w = c - '0';
    v = v * 16 + w;
  }
  return v;
}

typedef struct {
  char **line;
  int n, cap;
} lines_t;

static void lines_push(lines_t *L, char *s) {
  if (L->n == L->cap) {
    L->cap = L->cap ? 2 * L->cap : 1024;
    L->line = (char **)realloc(L->line, sizeof(char *) * L->cap);
  }
  L->line[L->n++] = s;
}

/* k-th token (0-based) of s split on single spaces; returns its length */
static size_t token(const char *s, int k, const char **beg) {
  const char *p = s;
  for (int i = 0; i < k; ++i) {
    const char *q = strchr(p, ' ');
    if (!q) {
      *beg = p + strlen(p);
      return 0;
    }
    p = q + 1;
  }
  const char *q = strchr(p, ' ');
  *beg = p;
  return q ? (size_t)(q - p) : strlen(p);
}

/* Text between the second '(' and the next ')' (betweenSecBrackets). */
static const char *second_bracket(const char *s, size_t *len) {
  const char *a = strchr(s, '(');
  if (!a) return NULL;
  const char *b = strchr(a + 1, '(');
  if (!b) return NULL;
  const char *c = strchr(b + 1, ')');
  *len = c ? (size_t)(c - b - 1) : strlen(b + 1);
  return b + 1;
}

static int geometry(om_mesh *m);

static void *xcalloc(size_t n, size_t s) {
  void *p = calloc(n ? n : 1, s);
  if (!p) {
    fprintf(stderr, "mstoracle: out of memory\n");
    abort();
  }
  return p;
}

static om_mesh *mesh_alloc(int nN, int nC, int nF) {
  om_mesh *m = (om_mesh *)xcalloc(1, sizeof(om_mesh));
  m->n_nodes = nN;
  m->n_cells = nC;
  m->n_faces = nF;
  m->node_xy = (double *)xcalloc((size_t)2 * nN, 8);
  m->face_nodes = (int *)xcalloc((size_t)2 * nF, 4);
  m->face_cells = (int *)xcalloc((size_t)2 * nF, 4);
  m->face_type = (int *)xcalloc(nF, 4);
  for (int i = 0; i < 2 * nF; ++i) m->face_cells[i] = -1;
  return m;
}

int om_mesh_read(const char *path, om_mesh **out) {
  *out = NULL;
  FILE *f = fopen(path, "rb");
  if (!f) return OM_EINVAL;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *buf = (char *)xcalloc((size_t)sz + 2, 1);
  if (fread(buf, 1, (size_t)sz, f) != (size_t)sz) {
    fclose(f);
    free(buf);
    return OM_EINVAL;
  }
  fclose(f);
  /* split lines, drop '\r' (the reference ran under Windows text mode) */
  lines_t hdr = {0}, dat = {0};
  lines_push(&dat, (char *)""); /* the data stream starts with "\n" */
  char *p = buf;
  while (*p) {
    char *e = strchr(p, '\n');
    if (e) *e = 0;
    size_t n = strlen(p);
    while (n && p[n - 1] == '\r') p[--n] = 0;
    if (p[0] == '(' || p[0] == ')') lines_push(&hdr, p);
    else lines_push(&dat, p);
    if (!e) break;
    p = e + 1;
  }
  int nN = -1, nC = -1, nF = -1, nI = 0;
  int flagNode = 0, flagFace = 0, di = 0, rc = OM_OK;
  om_mesh *m = NULL;
  int *zones = NULL, nz = 0;
  /* totals (10 (0 1 N 0 D)) (12 (0 ..)) (13 (0 ..)): the reference allocates
   * its arrays when it meets them; every shipped file gives each total
   * before the section that needs it, so a pre-pass is equivalent. */
  for (int h = 0; h < hdr.n; ++h) {
    const char *s = hdr.line[h];
    size_t bl;
    if (strlen(s) < 3 || s[1] != '1') continue;
    const char *br = second_bracket(s, &bl);
    if (!br || br[0] != '0') continue;
    const char *t;
    size_t tl = token(br, 2, &t);
    if (t > br + bl) continue;
    if (t + tl > br + bl) tl = (size_t)(br + bl - t);
    int v = hex_token(t, tl);
    if (s[2] == '0') nN = v;
    if (s[2] == '2') nC = v;
    if (s[2] == '3') nF = v;
  }
  if (nN <= 0 || nC <= 0 || nF <= 0) rc = OM_EMESH;
  else m = mesh_alloc(nN, nC, nF);
  for (int h = 0; h < hdr.n && rc == OM_OK; ++h) {
    const char *s = hdr.line[h];
    size_t sl = strlen(s);
    char c1 = sl > 1 ? s[1] : 0, c2 = sl > 2 ? s[2] : 0;
    if (c1 != '1') continue; /* names, dimension, zone table (39 ..) */
    size_t bl;
    const char *br = second_bracket(s, &bl);
    if (!br) continue;
    char inb[256];
    if (bl >= sizeof inb) bl = sizeof inb - 1;
    memcpy(inb, br, bl);
    inb[bl] = 0;
    if (inb[0] == '0') continue; /* totals, handled above */
    if (c2 != '0' && c2 != '3') continue;
    if (c2 == '0') { /* node section: one line consumed, then coordinates */
      di++;
      for (; flagNode < nN; ++flagNode) {
        if (di >= dat.n) {
          rc = OM_EMESH;
          break;
        }
        const char *ln = dat.line[di++];
        for (int d = 0; d < 2; ++d) {
          const char *t;
          size_t tl = token(ln, d, &t);
          char num[64];
          if (tl == 0 || tl >= sizeof num) {
            rc = OM_EMESH;
            break;
          }
          memcpy(num, t, tl);
          num[tl] = 0;
          m->node_xy[2 * flagNode + d] = strtod(num, NULL);
        }
        if (rc) break;
      }
    } else { /* face zone (13 (id start end type nodes)( */
      int v[5];
      for (int k = 0; k < 5; ++k) {
        const char *t;
        size_t tl = token(inb, k, &t);
        v[k] = hex_token(t, tl);
      }
      zones = (int *)realloc(zones, sizeof(int) * 4 * (nz + 1));
      zones[4 * nz] = v[0];
      zones[4 * nz + 1] = v[1];
      zones[4 * nz + 2] = v[2];
      zones[4 * nz + 3] = v[3];
      nz++;
      if (v[3] == 2) nI = v[2];
      if (v[4] != 2 || v[2] > nF) {
        rc = OM_EMESH;
        break;
      }
      for (; flagFace < v[2]; ++flagFace) {
        if (di >= dat.n) {
          rc = OM_EMESH;
          break;
        }
        const char *ln = dat.line[di++];
        int ids[4];
        int ntok = (v[3] == 2) ? 4 : 3;
        for (int k = 0; k < ntok; ++k) {
          const char *t;
          size_t tl = token(ln, k, &t);
          ids[k] = hex_token(t, tl) - 1;
        }
        if (ids[0] < 0 || ids[0] >= nN || ids[1] < 0 || ids[1] >= nN ||
            ids[2] < 0 || ids[2] >= nC ||
            (v[3] == 2 && (ids[3] < 0 || ids[3] >= nC))) {
          rc = OM_EMESH;
          break;
        }
        m->face_nodes[2 * flagFace] = ids[0];
        m->face_nodes[2 * flagFace + 1] = ids[1];
        m->face_cells[2 * flagFace] = ids[2];
        m->face_cells[2 * flagFace + 1] = (v[3] == 2) ? ids[3] : -1;
        m->face_type[flagFace] = v[3];
      }
    }
  }
  free(hdr.line);
  free(dat.line);
  free(buf);
  if (rc == OM_OK && (!m || flagNode != nN || flagFace != nF || nz == 0))
    rc = OM_EMESH;
  if (rc != OM_OK) {
    free(zones);
    if (m) om_mesh_free(m);
    return rc;
  }
  m->n_int_faces = nI;
  m->n_zones = nz;
  m->zone = zones;
  rc = geometry(m);
  if (rc != OM_OK) {
    om_mesh_free(m);
    return rc;
  }
  *out = m;
  return OM_OK;
}

int om_mesh_from_arrays(int n_nodes, const double *node_xy, int n_cells,
                        int n_faces, const int *face_nodes,
                        const int *face_cells, int n_zones, const int *zones,
                        om_mesh **out) {
  return om_mesh_from_arrays_periodic(n_nodes, node_xy, n_cells, n_faces,
                                      face_nodes, face_cells, n_zones, zones,
                                      NULL, out);
}

int om_mesh_from_arrays_periodic(int n_nodes, const double *node_xy,
                                 int n_cells, int n_faces,
                                 const int *face_nodes, const int *face_cells,
                                 int n_zones, const int *zones,
                                 const double *c1_shift, om_mesh **out) {
  *out = NULL;
  if (n_nodes <= 0 || n_cells <= 0 || n_faces <= 0 || n_zones <= 0)
    return OM_EINVAL;
  om_mesh *m = mesh_alloc(n_nodes, n_cells, n_faces);
  memcpy(m->node_xy, node_xy, sizeof(double) * 2 * n_nodes);
  memcpy(m->face_nodes, face_nodes, sizeof(int) * 2 * n_faces);
  memcpy(m->face_cells, face_cells, sizeof(int) * 2 * n_faces);
  m->n_zones = n_zones;
  if (c1_shift) {
    m->face_shift = (double *)xcalloc((size_t)2 * n_faces, 8);
    memcpy(m->face_shift, c1_shift, sizeof(double) * 2 * n_faces);
  }
  m->zone = (int *)xcalloc((size_t)4 * n_zones, 4);
  memcpy(m->zone, zones, sizeof(int) * 4 * n_zones);
  m->n_int_faces = 0;
  for (int z = 0; z < n_zones; ++z) {
    int s = zones[4 * z + 1] - 1, e = zones[4 * z + 2], t = zones[4 * z + 3];
    if (s < 0 || e > n_faces || s > e) {
      om_mesh_free(m);
      return OM_EINVAL;
    }
    if (t == 2) m->n_int_faces = e;
    for (int i = s; i < e; ++i) {
      m->face_type[i] = t;
      if (t != 2) m->face_cells[2 * i + 1] = -1;
    }
  }
  int rc = geometry(m);
  if (rc != OM_OK) {
    om_mesh_free(m);
    return rc;
  }
  *out = m;
  return OM_OK;
}

void om_mesh_free(om_mesh *m) {
  if (!m) return;
  free(m->zone);
  free(m->node_xy);
  free(m->face_nodes);
  free(m->face_cells);
  free(m->face_type);
  free(m->face_ctr);
  free(m->face_dir);
  free(m->face_area);
  free(m->face_eta0);
  free(m->face_dac);
  free(m->face_flag);
  free(m->cell_ptr);
  free(m->cell_faces);
  free(m->cell_nb);
  free(m->cell_dof);
  free(m->cell_eta0c);
  free(m->cell_ctr);
  free(m->cell_vol);
  free(m->inner);
  free(m->bond1);
  free(m->bond2);
  free(m->face_shift);
  free(m);
}

static double norm2(double a, double b) { return sqrt(a * a + b * b); }

/* shift of face f's c1 image (zero without periodic images) */
static double shift_of(const om_mesh *m, int f, int d) {
  return m->face_shift ? m->face_shift[2 * f + d] : 0.0;
}
/* centre of face f as seen from cell c: the c1 side of a periodic face
 * sees it translated back into its own frame */
static double face_ctr_from(const om_mesh *m, int f, int c, int d) {
  double x = m->face_ctr[2 * f + d];
  if (m->face_shift && m->face_cells[2 * f] != c) x = x - m->face_shift[2 * f + d];
  return x;
}

/* Geometry and derived connectivity: MshBlock.cpp:238-259 (cell lists),
 * Face::setCenter (Face.cpp:8-19), Cell::setCenter/setVolume
 * (Cell.cpp:6-50), orientation flags (MshBlock.cpp:281-305),
 * directOfNbFaces (:307-318), eta0 (Face.cpp:62-69, MshBlock.cpp:319-334),
 * boundary cell lists (:370-406). */
static int geometry(om_mesh *m) {
  const int nC = m->n_cells, nF = m->n_faces;
  /* per-cell face lists in face order: c0 then c1 of each face */
  m->cell_ptr = (int *)xcalloc((size_t)nC + 1, 4);
  for (int i = 0; i < nF; ++i) {
    int c0 = m->face_cells[2 * i], c1 = m->face_cells[2 * i + 1];
    if (c0 < 0 || c0 >= nC || c1 >= nC) return OM_EMESH;
    m->cell_ptr[c0 + 1]++;
    if (c1 >= 0) m->cell_ptr[c1 + 1]++;
  }
  for (int c = 0; c < nC; ++c) m->cell_ptr[c + 1] += m->cell_ptr[c];
  int tot = m->cell_ptr[nC];
  m->cell_faces = (int *)xcalloc(tot, 4);
  m->cell_nb = (int *)xcalloc(tot, 4);
  m->cell_dof = (double *)xcalloc((size_t)2 * tot, 8);
  m->cell_eta0c = (double *)xcalloc(tot, 8);
  int *fill = (int *)xcalloc(nC, 4);
  for (int i = 0; i < nF; ++i) {
    int c0 = m->face_cells[2 * i], c1 = m->face_cells[2 * i + 1];
    int k0 = m->cell_ptr[c0] + fill[c0]++;
    m->cell_faces[k0] = i;
    m->cell_nb[k0] = (c1 >= 0) ? c1 : c0;
    if (c1 >= 0) {
      int k1 = m->cell_ptr[c1] + fill[c1]++;
      m->cell_faces[k1] = i;
      m->cell_nb[k1] = c0;
    }
  }
  free(fill);
  /* faces */
  m->face_ctr = (double *)xcalloc((size_t)2 * nF, 8);
  m->face_dir = (double *)xcalloc((size_t)2 * nF, 8);
  m->face_area = (double *)xcalloc(nF, 8);
  m->face_eta0 = (double *)xcalloc(nF, 8);
  m->face_dac = (int *)xcalloc(nF, 4);
  m->face_flag = (uint8_t *)xcalloc((size_t)2 * nF, 1);
  for (int i = 0; i < nF; ++i) {
    const double *a = m->node_xy + 2 * m->face_nodes[2 * i];
    const double *b = m->node_xy + 2 * m->face_nodes[2 * i + 1];
    for (int d = 0; d < 2; ++d) {
      double s = 0.0;
      s += a[d];
      s += b[d];
      m->face_ctr[2 * i + d] = s / 2.0;
    }
    double f0 = a[0] - b[0], f1 = a[1] - b[1];
    m->face_area[i] = norm2(f0, f1);
    m->face_dir[2 * i] = -f1;
    m->face_dir[2 * i + 1] = f0;
  }
  /* cells: centre = mean of face centres, volume by Heron */
  m->cell_ctr = (double *)xcalloc((size_t)2 * nC, 8);
  m->cell_vol = (double *)xcalloc(nC, 8);
  for (int c = 0; c < nC; ++c) {
    int b = m->cell_ptr[c], n = m->cell_ptr[c + 1] - b;
    for (int d = 0; d < 2; ++d) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += face_ctr_from(m, m->cell_faces[b + k], c, d);
      m->cell_ctr[2 * c + d] = s / (double)n;
    }
#define LEN(k) norm2(m->face_dir[2 * m->cell_faces[b + (k)]], \
                     m->face_dir[2 * m->cell_faces[b + (k)] + 1])
#define FC(k, d) face_ctr_from(m, m->cell_faces[b + (k)], c, (d))
    double vol = 0.0;
    if (n == 3) {
      double l0 = LEN(0), l1 = LEN(1), l2 = LEN(2);
      double s = 0.5 * (l0 + l1 + l2);
      vol = sqrt(s * (s - l0) * (s - l1) * (s - l2));
    } else if (n == 4) {
      double v1x = FC(0, 0) - FC(1, 0), v1y = FC(0, 1) - FC(1, 1);
      double v2x = FC(2, 0) - FC(3, 0), v2y = FC(2, 1) - FC(3, 1);
      int a0, a1, b0, b1;
      double mid;
      if (fabs(v1x * v2y - v2x * v1y) < EOR2_) {
        mid = 2 * norm2(FC(0, 0) - FC(1, 0), FC(0, 1) - FC(1, 1));
        a0 = 0, a1 = 1, b0 = 2, b1 = 3;
      } else {
        mid = 2 * norm2(FC(0, 0) - FC(2, 0), FC(0, 1) - FC(2, 1));
        a0 = 0, a1 = 2, b0 = 1, b1 = 3;
      }
      double la0 = LEN(a0), la1 = LEN(a1), lb0 = LEN(b0), lb1 = LEN(b1);
      double s = 0.5 * (la0 + la1 + mid);
      vol = sqrt(s * (s - la0) * (s - la1) * (s - mid));
      double s2 = 0.5 * (lb0 + lb1 + mid);
      vol += sqrt(s2 * (s2 - lb0) * (s2 - lb1) * (s2 - mid));
    } else {
      return OM_EMESH; /* the 2D reader handles triangles and quads only */
    }
#undef LEN
#undef FC
    m->cell_vol[c] = vol;
  }
  /* orientation flags */
  for (int i = 0; i < nF; ++i) {
    int c0 = m->face_cells[2 * i];
    const double *dv = m->face_dir + 2 * i;
    double t = dv[0] * (m->face_ctr[2 * i] - m->cell_ctr[2 * c0]);
    t += dv[1] * (m->face_ctr[2 * i + 1] - m->cell_ctr[2 * c0 + 1]);
    if (t < 0) {
      m->face_dac[i] = -1;
      for (int d = 0; d < 2; ++d) m->face_flag[2 * i + d] = (-1.0 * dv[d] >= 0);
    } else {
      m->face_dac[i] = 1;
      for (int d = 0; d < 2; ++d) m->face_flag[2 * i + d] = !(1.0 * dv[d] >= 0);
    }
  }
  /* outward area vector per cell-face */
  for (int c = 0; c < nC; ++c)
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      int f = m->cell_faces[k];
      double s = (double)((m->face_cells[2 * f] == c) ? m->face_dac[f]
                                                      : -m->face_dac[f]);
      m->cell_dof[2 * k] = s * m->face_dir[2 * f];
      m->cell_dof[2 * k + 1] = s * m->face_dir[2 * f + 1];
    }
  /* eta0 */
  for (int i = 0; i < nF; ++i) {
    int c0 = m->face_cells[2 * i], c1 = m->face_cells[2 * i + 1];
    if (c1 >= 0) {
      const double *fc = m->face_ctr + 2 * i;
      double x1 = m->cell_ctr[2 * c1] + shift_of(m, i, 0);
      double y1 = m->cell_ctr[2 * c1 + 1] + shift_of(m, i, 1);
      double n1 = norm2(x1 - fc[0], y1 - fc[1]);
      double n0 = norm2(m->cell_ctr[2 * c0] - fc[0], m->cell_ctr[2 * c0 + 1] - fc[1]);
      m->face_eta0[i] = n1 / (n0 + n1);
    } else {
      m->face_eta0[i] = 1;
    }
  }
  for (int c = 0; c < nC; ++c)
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      int f = m->cell_faces[k];
      m->cell_eta0c[k] = (m->face_cells[2 * f] == c) ? m->face_eta0[f]
                                                      : 1 - m->face_eta0[f];
    }
  /* boundary cell lists */
  uint8_t *flag = (uint8_t *)xcalloc(nC, 1);
  m->bond1 = (int *)xcalloc(nC, 4);
  m->bond2 = (int *)xcalloc(nC, 4);
  m->inner = (int *)xcalloc(nC, 4);
  m->n_bond1 = m->n_bond2 = m->n_inner = 0;
  for (int i = 0; i < nF; ++i)
    if (m->face_type[i] != 2) {
      int c0 = m->face_cells[2 * i];
      if (!flag[c0]) {
        m->bond1[m->n_bond1++] = c0;
        flag[c0] = 1;
      }
    }
  for (int b = 0; b < m->n_bond1; ++b) {
    int c = m->bond1[b];
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      int nb = m->cell_nb[k];
      if (!flag[nb]) {
        m->bond2[m->n_bond2++] = nb;
        flag[nb] = 1;
      }
    }
  }
  for (int c = 0; c < nC; ++c)
    if (!flag[c]) m->inner[m->n_inner++] = c;
  free(flag);
  return OM_OK;
}

/* ------------------------------------------------------------------ */
/* solver: RhoSolver.cpp                                               */
/* ------------------------------------------------------------------ */
/* inviscid wall / symmetry ghost: momentum mirrored about the face,
 * RhoSolver.cpp:150-160 */
static void mirror(const double *dir, const double in[4], double out[4]) {
  double nrm = norm2(dir[0], dir[1]);
  double n0 = dir[0] / nrm, n1 = dir[1] / nrm;
  double t = n0 * in[1];
  t += n1 * in[2];
  out[0] = in[0];
  out[1] = in[1] - 2 * n0 * t;
  out[2] = in[2] - 2 * n1 * t;
  out[3] = in[3];
}

/* Q + G (x_f - x_c), G as [2][4] */
static void recon(const double q[4], const double *g, const double *xf,
                  const double *xc, double out[4]) {
  double r0 = xf[0] - xc[0], r1 = xf[1] - xc[1];
  for (int k = 0; k < 4; ++k) {
    double s = g[k] * r0;
    s += g[4 + k] * r1;
    out[k] = q[k] + s;
  }
}

void om_gradient(const om_mesh *m, const double *q, double *faceq,
                 double *grad) {
  const int nI = m->n_int_faces, nF = m->n_faces;
  for (int i = 0; i < nI; ++i) {
    const double e = m->face_eta0[i];
    const double *q0 = q + 4 * m->face_cells[2 * i];
    const double *q1 = q + 4 * m->face_cells[2 * i + 1];
    for (int k = 0; k < 4; ++k) faceq[4 * i + k] = e * q0[k] + (1 - e) * q1[k];
  }
  for (int i = (nI > 0 ? nI - 1 : 0); i < nF; ++i)
    for (int k = 0; k < 4; ++k)
      faceq[4 * i + k] = q[4 * m->face_cells[2 * i] + k];
  for (int c = 0; c < m->n_cells; ++c) {
    double g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const double *fq = faceq + 4 * m->cell_faces[k];
      for (int d = 0; d < 2; ++d)
        for (int j = 0; j < 4; ++j) g[4 * d + j] += fq[j] * m->cell_dof[2 * k + d];
    }
    for (int j = 0; j < 8; ++j) grad[8 * c + j] = g[j] / m->cell_vol[c];
  }
}

void om_face_flux(const om_mesh *m, const om_params *p, const double *q,
                  const double *grad, double *F) {
  flux_fn fl = (p->flux == OM_ROE) ? om_roe_flux : om_ausm_flux;
  const int second = (p->order == 2);
  for (int z = 0; z < m->n_zones; ++z) {
    const int type = m->zone[4 * z + 3];
    const int s = m->zone[4 * z + 1] - 1, e = m->zone[4 * z + 2];
    for (int i = s; i < e; ++i) {
      const int c0 = m->face_cells[2 * i], c1 = m->face_cells[2 * i + 1];
      const uint8_t *flag = m->face_flag + 2 * i;
      const double *xf = m->face_ctr + 2 * i;
      double a[4], b[4];
      double *Fi = F + 8 * i;
      switch (type) {
        case 2: /* interior, RhoSolver.cpp:99-118 / :243-260 */
          if (second) {
            recon(q + 4 * c0, grad + 8 * c0, xf, m->cell_ctr + 2 * c0, a);
            recon(q + 4 * c1, grad + 8 * c1, xf, m->cell_ctr + 2 * c1, b);
          } else {
            memcpy(a, q + 4 * c0, 32);
            memcpy(b, q + 4 * c1, 32);
          }
          for (int d = 0; d < 2; ++d) {
            if (flag[d]) fl(a, b, d, Fi + 4 * d);
            else fl(b, a, d, Fi + 4 * d);
          }
          break;
        case 10: /* inlet, fixed state, :119-139 / :262-282 */
          if (second) recon(q + 4 * c0, grad + 8 * c0, xf, m->cell_ctr + 2 * c0, a);
          else memcpy(a, q + 4 * c0, 32);
          for (int d = 0; d < 2; ++d) {
            if (flag[d]) fl(a, p->inlet_q, d, Fi + 4 * d);
            else fl(p->inlet_q, a, d, Fi + 4 * d);
          }
          break;
        case 3: /* inviscid wall, :140-181 / :283-319 */
          if (second) recon(q + 4 * c0, grad + 8 * c0, xf, m->cell_ctr + 2 * c0, a);
          else memcpy(a, q + 4 * c0, 32);
          mirror(m->face_dir + 2 * i, a, b);
          for (int d = 0; d < 2; ++d) {
            if (flag[d]) fl(a, b, d, Fi + 4 * d);
            else fl(b, a, d, Fi + 4 * d);
          }
          break;
        case 7: /* symmetry, :182-213; 2nd order reconstructs the ghost
                   (density, energy) but mirrors the cell momentum, :320-350 */
          memcpy(a, q + 4 * c0, 32);
          if (second) {
            double r[4];
            recon(q + 4 * c0, grad + 8 * c0, xf, m->cell_ctr + 2 * c0, r);
            double mm[4];
            mirror(m->face_dir + 2 * i, a, mm);
            b[0] = r[0];
            b[1] = mm[1];
            b[2] = mm[2];
            b[3] = r[3];
          } else {
            mirror(m->face_dir + 2 * i, a, b);
          }
          for (int d = 0; d < 2; ++d) {
            if (flag[d]) fl(a, b, d, Fi + 4 * d);
            else fl(b, a, d, Fi + 4 * d);
          }
          break;
        case 5: /* outlet: zero-gradient, no flag test, :214-228 */
          memcpy(a, q + 4 * c0, 32);
          for (int d = 0; d < 2; ++d) fl(a, a, d, Fi + 4 * d);
          break;
        default:
          break;
      }
    }
  }
}

void om_gather(const om_mesh *m, const double *F, double *R) {
#pragma omp parallel for schedule(static)
  for (int c = 0; c < m->n_cells; ++c) {
    double r[4] = {0, 0, 0, 0};
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      const double *Ff = F + 8 * m->cell_faces[k];
      for (int d = 0; d < 2; ++d) {
        double s = m->cell_dof[2 * k + d];
        for (int j = 0; j < 4; ++j) r[j] += s * Ff[4 * d + j];
      }
    }
    for (int j = 0; j < 4; ++j) R[4 * c + j] = r[j];
  }
}

void om_solve(const om_mesh *m, const om_params *p, const double *q,
              double dt, double *qnew, double *R) {
  double *F = (double *)xcalloc((size_t)8 * m->n_faces, 8);
  double *grad = NULL, *faceq = NULL;
  if (p->order == 2) {
    grad = (double *)xcalloc((size_t)8 * m->n_cells, 8);
    faceq = (double *)xcalloc((size_t)4 * m->n_faces, 8);
    om_gradient(m, q, faceq, grad);
  }
  om_face_flux(m, p, q, grad, F);
  double *Rl = R ? R : (double *)xcalloc((size_t)4 * m->n_cells, 8);
  om_gather(m, F, Rl);
  for (int c = 0; c < m->n_cells; ++c) {
    double f = dt / m->cell_vol[c];
    for (int j = 0; j < 4; ++j) qnew[4 * c + j] = q[4 * c + j] - f * Rl[4 * c + j];
  }
  if (!R) free(Rl);
  free(F);
  free(grad);
  free(faceq);
}

void om_linf_change(int n_cells, const double *qold, const double *qnew,
                    double res[4]) {
  for (int j = 0; j < 4; ++j) res[j] = 0;
  for (int c = 0; c < n_cells; ++c)
    for (int j = 0; j < 4; ++j) {
      double r = fabs(qnew[4 * c + j] - qold[4 * c + j]) / qold[4 * c + j];
      if (res[j] < r) res[j] = r;
    }
}
