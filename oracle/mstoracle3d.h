/* CPU restatement of the 3D density-based residual path (test
 * infrastructure only: the checker of the product's mst_ctx3d_* entry
 * points; nothing here is linked into the product).
 *
 * The reference's 3D path cannot run (its thermodynamics are 2D-only,
 * work/FUNCTION.cpp:3-18, AllData.cpp:95-98; its 3D cell volume and quad
 * face area are wrong, mesh/Cell.cpp:52-59, mesh/Face.cpp:30-36), so this is
 * the reference's 2D density path (rhoSolver/RhoSolver.cpp:37-453) carried
 * to three dimensions with those defects corrected, as the 2D corrected
 * mode does:
 *   geometry   face centre = mean of its nodes, area vector 1/2 (n1-n0) x
 *              (n2-n0) (triangle) or 1/2 (n2-n0) x (n3-n1) (quadrilateral),
 *              oriented out of c0; cell centre = mean of its face centres
 *              (Cell.cpp:6-14); volume by the divergence theorem;
 *              periodic faces carry the shift of c1's frame
 *   gradient   Green-Gauss of the conserved state with eta0-weighted face
 *              values (RhoSolver.cpp:430-453), boundary faces the cell value
 *   flux       split-axis: for each axis d the 1D Roe flux (SolverRoe.cpp
 *              :70-123, Roe averages with D = sqrt(rho_R/rho_L), absolute
 *              entropy fix 0.125) between the states ordered along d, its
 *              |A| dQ in the closed wave-strength form (equal to R|L|R^-1 dQ
 *              for the Roe-averaged state); reconstruction unlimited or
 *              edge-based MUSCL with minmod / van Leer / van Albada; the
 *              laminar viscous term; boundary ghosts: inlet, outlet, wall
 *              (mirror, or no-slip when viscous), symmetry
 *   residual   R_c = sum over the cell's faces (ascending face id) of
 *              sum_d S_out,d F_d
 *   update     explicit RK2 with the global CFL step of the 2D path.
 * All arithmetic FP64 in the order of the CUDA exact path; compile with
 * -ffp-contract=off. */
#ifndef MSTORACLE3D_H
#define MSTORACLE3D_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n_nodes, n_cells, n_faces;
  const double *node_xyz;     /* [nN][3] */
  const int *face_ptr;        /* [nF+1] into face_nodes */
  const int *face_nodes;      /* 3 or 4 nodes per face, in c0's frame */
  const int *face_cells;      /* [nF][2], c1 = -1 on boundary faces */
  const int *face_type;       /* [nF] Fluent zone type (2 interior, 3 wall,
                                 5 outlet, 7 symmetry, 10 inlet) */
  const double *c1_shift;     /* [nF][3] x(c0 frame) - x(c1 frame), or NULL */
} om3_input;

typedef struct {
  int n_cells, n_faces;
  int *face_cells, *face_kind;   /* kind: 0 interior, 1 inlet, 2 wall,
                                    3 symmetry, 4 outlet, 5 none */
  double *face_ctr, *face_dir;   /* [nF][3]; dir points out of c0 */
  double *r0, *r1;               /* [nF][3] x_f - x_c0, x_f - x_c1 (c1 frame) */
  double *eta;                   /* [nF] |r1| / (|r0| + |r1|), 1 on boundary */
  double *cell_ctr, *cell_vol;   /* [nC][3], [nC] */
  int *cell_ptr, *cell_faces, *cell_nb;  /* CSR, faces ascending; nb = the
                                            other cell or -1 on boundary */
  double *cell_dir;              /* [tot][3] area vector out of the cell */
  double *cell_w;                /* [tot][2] face-value weights (self, nb) */
} om3_mesh;

int om3_build(const om3_input *in, om3_mesh *m);
void om3_free(om3_mesh *m);

enum { OM3_LIM_NONE = 0, OM3_LIM_MINMOD = 1, OM3_LIM_VANLEER = 2, OM3_LIM_VANALBADA = 3 };

typedef struct {
  int order;     /* 1 or 2 */
  int limiter;   /* OM3_LIM_* (2nd order) */
  int viscous;
  double mu, lam, kappa, cv;
  double inlet[5];
} om3_params;

/* grad [nC][3][5]: d/dx_d of component j at [c][d][j] */
void om3_gradient(const om3_mesh *m, const double *q, double *grad);
/* F [nF][3][5]: the flux of each axis of every face (grad NULL: 1st order) */
void om3_face_flux(const om3_mesh *m, const om3_params *p, const double *q,
                   const double *grad, double *F);
/* R [nC][5] */
void om3_gather(const om3_mesh *m, const double *F, double *R);
/* R of state q (gradient, fluxes and gather) */
void om3_residual(const om3_mesh *m, const om3_params *p, const double *q, double *R);
/* global CFL step: min over cells of cfl V / (0.5 sum_k (|u.S_k| + a|S_k|)) */
double om3_dt(const om3_mesh *m, const double *q, double cfl);
/* nsteps RK2 steps of q in place at CFL cfl (dt of each step from its
 * state, cut to reach t_end when t_end > 0); *time advanced */
int om3_rk2(const om3_mesh *m, const om3_params *p, double *q, int nsteps, double cfl,
            double t_end, double *time);
/* sum 1/2 |m|^2 / rho V over the cells and sum V */
void om3_kinetic_energy(const om3_mesh *m, const double *q, double *ke, double *vol);

#ifdef __cplusplus
}
#endif
#endif
