/* CPU restatement of MST-CFD's density-based finite-volume residual path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA path is checked
 * against; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it, and only as the checker or the timed CPU baseline, never
 * as a product code path.
 *
 * Parity pinning: every function below restates a reference function
 * (file:line cited at each definition, paths within MST-CFD/) and is
 * checked bit-for-bit against the reference itself, compiled here from its
 * own sources into oracle/_ref (oracle/ref/build_ref.sh), on the eight
 * shipped meshes and on generated meshes (tests/test_oracle_vs_ref.py).
 * The reference's Eigen arithmetic is pinned to the project's Eigen-subset
 * shim (oracle/ref/eigen_shim), whose reduction order and 4x4 inverse this
 * file follows; real Eigen is not installed, so parity with a particular
 * Eigen build is unpinned.
 *
 * Layout: all arrays are flat, row-major, little endian; cell states are
 * AoS [n_cells][4] = (rho, rho*u, rho*v, E); face flux matrices are
 * [n_faces][2][4] (axis-major: F[f][d][m]); gradients [n_cells][2][4].
 */
#ifndef MSTORACLE_H
#define MSTORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct om_mesh {
  int n_nodes, n_cells, n_faces, n_int_faces, n_zones;
  int n_inner, n_bond1, n_bond2;
  /* zones: [n_zones][4] = (zone id, first face (1-based), last face, type) */
  int *zone;
  double *node_xy;     /* [n_nodes][2] */
  int *face_nodes;     /* [n_faces][2] (0-based) */
  int *face_cells;     /* [n_faces][2] (c1 = -1 on boundary faces) */
  int *face_type;      /* [n_faces] zone type of the face */
  double *face_ctr;    /* [n_faces][2] */
  double *face_dir;    /* [n_faces][2] area vector (-(y0-y1), x0-x1) */
  double *face_area;   /* [n_faces] */
  double *face_eta0;   /* [n_faces] */
  int *face_dac;       /* [n_faces] directAndCells: +1 or -1 */
  uint8_t *face_flag;  /* [n_faces][2] flagLeftRight */
  int *cell_ptr;       /* [n_cells+1] CSR into the per-cell-face arrays */
  int *cell_faces;     /* face ids, ascending (file order) */
  int *cell_nb;        /* neighbour cell per cell-face (itself on boundary) */
  double *cell_dof;    /* [total][2] outward area vector per cell-face */
  double *cell_eta0c;  /* [total] */
  double *cell_ctr;    /* [n_cells][2] */
  double *cell_vol;    /* [n_cells] */
  int *inner, *bond1, *bond2;
  /* periodic images (project extension; NULL for reference meshes):
   * [n_faces][2] translation mapping cell c1's coordinates into the frame
   * of the face and of c0 */
  double *face_shift;
} om_mesh;

/* status codes (match the product's C ABI) */
#define OM_OK 0
#define OM_EINVAL 1
#define OM_EMESH 2

/* Reads the Fluent ASCII subset MshBlock accepts (mesh/MshBlock.cpp:75-432). */
int om_mesh_read(const char *path, om_mesh **out);
/* Builds the same mesh from raw arrays (the product's mesh generators):
 * zones [n_zones][4] as above; face_cells c1 = -1 on boundary faces. */
int om_mesh_from_arrays(int n_nodes, const double *node_xy, int n_cells,
                        int n_faces, const int *face_nodes,
                        const int *face_cells, int n_zones, const int *zones,
                        om_mesh **out);
/* Same, with periodic image shifts (may be NULL). */
int om_mesh_from_arrays_periodic(int n_nodes, const double *node_xy,
                                 int n_cells, int n_faces,
                                 const int *face_nodes, const int *face_cells,
                                 int n_zones, const int *zones,
                                 const double *c1_shift, om_mesh **out);
void om_mesh_free(om_mesh *m);

/* Flux schemes */
#define OM_AUSM 0
#define OM_ROE 1

typedef struct om_params {
  int flux;          /* OM_AUSM or OM_ROE */
  int order;         /* 1 or 2 */
  double inlet_q[4]; /* type-10 state (reference: CONST.h inlet macros) */
} om_params;

void om_default_params(om_params *p);
/* Reference inlet / initial state (CONST.h:70-83). */
void om_reference_inlet(double q[4]);

/* Riemann fluxes of one face along axis d (SolverAusm.cpp, SolverRoe.cpp). */
void om_ausm_flux(const double ql[4], const double qr[4], int d, double f[4]);
void om_roe_flux(const double ql[4], const double qr[4], int d, double f[4]);

/* Green-Gauss gradient of conserved Q (RhoSolver.cpp:430-453), incl. the
 * boundary loop starting at nInt-1.  faceq [n_faces][4], grad [n_cells][2][4]. */
void om_gradient(const om_mesh *m, const double *q, double *faceq,
                 double *grad);

/* Face flux matrices (RhoSolver.cpp:90-233 first order, :234-369 second
 * order).  grad may be NULL for order 1.  F [n_faces][2][4]. */
void om_face_flux(const om_mesh *m, const om_params *p, const double *q,
                  const double *grad, double *F);

/* Per-cell residual gather (RhoSolver.cpp:45-56).  R [n_cells][4]. */
void om_gather(const om_mesh *m, const double *F, double *R);

/* One RhoSolver::solve(): flux (+gradient), gather and the explicit update
 * Qnew = Qold - DT/V*R (RhoSolver.cpp:37-68).  R may be NULL. */
void om_solve(const om_mesh *m, const om_params *p, const double *q,
              double dt, double *qnew, double *R);

/* Time::goNextTimeStep residual: max over cells of |Qn-Qo|/Qo per
 * component, signed division as in time/Time.cpp:69-76. */
void om_linf_change(int n_cells, const double *qold, const double *qnew,
                    double res[4]);

/* ------------------------------------------------------------------ */
/* Project extensions with no reference counterpart (mstoracle_ext.c):  */
/* corrected boundary handling, TVD limiters, periodic images, CFL time */
/* steps and the two-stage Runge-Kutta update.  Each restates the       */
/* published method named at its definition, in the operation order of  */
/* the CUDA kernels (so the FP64-exact GPU path matches bit-for-bit).   */
/* ------------------------------------------------------------------ */
#define OM_LIM_NONE 0
#define OM_LIM_MINMOD 1
#define OM_LIM_VANLEER 2
#define OM_LIM_VANALBADA 3
#define OM_DT_FIXED 0
#define OM_DT_CFL_GLOBAL 1
#define OM_DT_CFL_LOCAL 2

typedef struct om_params_ext {
  int flux, order, limiter;
  int quirks;       /* 1: the reference's behaviour; 0: corrected */
  int rk2;          /* 0 forward Euler, 1 two-stage SSP Runge-Kutta */
  int dt_mode;      /* OM_DT_* */
  double dt, cfl;
  double inlet_q[4];
  int viscous;      /* laminar viscous term (order 2) */
  double mu, lam, kappa, cv;
  /* limiter freezing (limited 2nd order): phi [n_faces][2][4] the ratios
   * slope / (upwind difference) of each face side; phi_mode 0 off,
   * 1 record, 2 use (times the current upwind difference) */
  double *phi;
  int phi_mode;
  /* limited faces: a reconstructed side with non-positive density or
   * pressure takes its cell value (the implicit iterations set this) */
  int positivity;
} om_params_ext;

typedef struct om_norms {
  double linf[4], l2[4], mass, dt, time;
} om_norms;

void om_default_params_ext(om_params_ext *p);
void om_gradient_ext(const om_mesh *m, const double *q, int quirks,
                     double *grad);
void om_face_flux_ext(const om_mesh *m, const om_params_ext *p,
                      const double *q, const double *grad, double *F);
/* per-cell CFL step dt_c = cfl V / (0.5 sum_f (|u.n| + a|n|)); returns
 * the minimum (0 where the state is not physical) */
double om_spectral_dt(const om_mesh *m, const double *q, double cfl,
                      double *dt_cell);
/* nsteps time steps in place; *time is advanced; last = norms of the last
 * step (nullable) */
int om_step_ext(const om_mesh *m, const om_params_ext *p, double *q,
                int nsteps, double t_end, double *time, om_norms *last);

/* ------------------------------------------------------------------ */
/* sparse sweeps of lusolver/ (mstoracle_lu.c)                          */
/* ------------------------------------------------------------------ */
/* Scalar SparseSolverNUM::solveILUSGS (gs = 0) or solveGS (gs = 1) on the
 * system built by the ordered insertions (rows[i], cols[i], vals[i]) with
 * ops[i] = 0 setELE, 1 addELE.  x: initial guess in, solution out. */
/* ---- pressure-based SIMPLE (mstoracle_simple.c) ---- */
typedef struct om_simple_params {
  double dt;          /* 1 / STEP_TIME */
  double alpha_p;     /* SIMPLE_ALPHA_P: p += alpha_p p' */
  int n_inner;        /* SIMPLE_INTERVAL: SIMPLE iterations per step */
  int wall_smooth;    /* FLAG_WALLSMOOTH */
  double inlet[4];    /* face (p, u, v, T) on inlet (type 10) faces */
  double p_out;       /* face pressure on outlet (type 5) faces */
} om_simple_params;
void om_simple_default_params(om_simple_params *p);
/* (p, u, v, T) of conserved states, as Time::initialization forms them */
void om_q_to_puvt(int n, const double *q, double *puvt);
/* nsteps time steps; puvt [n_cells][4] and face [n_faces][4] in/out;
 * time_rows [nsteps][4], inner_rows [nsteps][n_inner][4] and gs_iters
 * [nsteps][n_inner][3] (u, v, p' solves) may be NULL */
int om_simple_step(const om_mesh *m, const om_simple_params *p, double *puvt,
                   double *face, int nsteps, double *time_rows, double *inner_rows,
                   int *gs_iters);

int om_lu_scalar(int gs, int dim, int n, const int *rows, const int *cols,
                 const int *ops, const double *vals, const double *b, double *x,
                 int *iterations);
/* Block SparseSolver<Matrix4d, Vector4d>::solveILU: vals [n][16] row-major
 * blocks (diagonal entries setD, below setL, above setU), b and x [dim][4]. */
int om_lu_block(int dim, int n, const int *rows, const int *cols,
                const double *vals, const double *b, double *x);

#ifdef __cplusplus
}
#endif
#endif
