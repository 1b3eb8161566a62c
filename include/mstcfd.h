/* mstcfd.h -- C ABI of the GB300 (sm_103a) density-based unstructured
 * finite-volume residual path.
 *
 * Drop-in boundary for MST-CFD's RhoSolver (rhoSolver/RhoSolver.h:14-56 in
 * the reference).  Every entry point returns an mst_status, never aborts and
 * never lets an exception cross the boundary.  Plain pointers and sizes
 * only.  The caller owns host buffers; a context owns its device buffers and
 * one CUDA stream.  One context per host thread; contexts are independent.
 *
 * Numbering: cells and faces keep the numbering of the .msh file (0-based);
 * any device-side renumbering is internal and invisible at this boundary.
 * States are AoS rows of 4 doubles (rho, rho*u, rho*v, E) with a caller
 * stride (in doubles, >= 4), so an array of the reference's VCTDIMU
 * (Eigen Matrix<double,4,1>, 32-byte stride) is passed as-is with stride 4.
 */
#ifndef MSTCFD_H
#define MSTCFD_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSTCFD_ABI_VERSION 1

typedef enum mst_status {
  MST_OK = 0,
  MST_EINVAL = 1,      /* bad argument */
  MST_EMESH = 2,       /* malformed or unsupported mesh */
  MST_ECUDA = 3,       /* CUDA runtime error (see mst_last_error) */
  MST_EDIVERGED = 4,   /* NaN or non-positive density/pressure */
  MST_ETIMEOUT = 5,    /* a bounded device wait gave up */
  MST_ENOMEM = 6,      /* host or device allocation failed */
  MST_EUNSUPPORTED = 7 /* option combination not built */
} mst_status;

/* Riemann flux (reference: CONST.h:10 RHOSOLVER) */
enum { MST_FLUX_AUSM = 0, MST_FLUX_ROE = 1 };
/* TVD limiter for 2nd order (none = the reference's unlimited scheme) */
enum {
  MST_LIMITER_NONE = 0,
  MST_LIMITER_MINMOD = 1,
  MST_LIMITER_VANLEER = 2,
  MST_LIMITER_VANALBADA = 3
};
/* Arithmetic of reconstruction + flux.  FP64_EXACT rounds every operation
 * like the reference (no fused multiply-add); FP64 allows FMA; FP32 runs
 * reconstruction and flux in float and keeps the state, the residual
 * accumulation and the norms in double. */
enum { MST_PREC_FP64_EXACT = 0, MST_PREC_FP64 = 1, MST_PREC_FP32 = 2 };
/* Time integration: one forward-Euler stage (RhoSolver.cpp:64) or the
 * two-stage SSP Runge-Kutta (Heun) scheme. */
enum { MST_TIME_EULER = 0, MST_TIME_RK2 = 1 };
/* Time step: fixed (RhoSolver::setDT), global CFL, or local (per-cell) CFL */
enum { MST_DT_FIXED = 0, MST_DT_CFL_GLOBAL = 1, MST_DT_CFL_LOCAL = 2 };

typedef struct mst_params {
  int flux;          /* MST_FLUX_* */
  int order;         /* 1 or 2 (reference: CONST.h:6 ACCURACY) */
  int limiter;       /* MST_LIMITER_* (order 2 only) */
  int precision;     /* MST_PREC_* */
  int time_scheme;   /* MST_TIME_* */
  int dt_mode;       /* MST_DT_* */
  double dt;         /* fixed step; reference default 1/STEP_TIME = 1/4000 */
  double cfl;        /* CFL number for the CFL modes */
  double inlet_q[4]; /* type-10 boundary state (reference: CONST.h:77-83) */
  /* 1 = reproduce the reference bit-for-bit, including its quirks (left/right
   * flags as MshBlock.cpp:281-305 sets them, boundary face values from
   * nInt-1, symmetry ghost of RhoSolver.cpp:320-350).  0 = corrected
   * behaviour (geometric left/right, boundary loops from nInt, 2nd-order
   * symmetry = mirrored reconstructed state, 2nd-order outlet =
   * reconstructed zero-gradient). */
  int reference_quirks;
  /* Laminar viscous term (order 2 only; the reference's updateViscid,
   * RhoSolver.cpp:371-429, restated with its defects corrected): stress
   * tau = mu (grad u + grad u^T) + lambda (div u) I, heat flux kappa grad T
   * with T = e / cv; walls become no-slip and adiabatic.  Defaults are
   * CONST.h's VISCIDMU, VISCIDLAMBDA, TEMPK and CV. */
  int viscous;
  double mu, lambda, kappa, cv;
  int reserved[6];
} mst_params;

/* Reference defaults: AUSM+, 1st order, FP64_EXACT, Euler, DT = 1/4000,
 * inlet state of CONST.h, quirks on, inviscid. */
void mst_params_default(mst_params *p);

/* ------------------------------------------------------------------ */
/* meshes                                                              */
/* ------------------------------------------------------------------ */
typedef struct mst_mesh mst_mesh;

/* Reads a Fluent ASCII 2D mesh (the subset of MshBlock::readMsh,
 * mesh/MshBlock.cpp:5-18, :75-432) and builds its geometry exactly as the
 * reference does (Face::setCenter Face.cpp:8-19, Cell::setCenter/setVolume
 * Cell.cpp:6-50, orientation flags MshBlock.cpp:281-305, directOfNbFaces
 * :307-318, eta0 :319-334).  Accepts CRLF or LF line ends. */
mst_status mst_mesh_read_msh(const char *path, mst_mesh **out);

typedef struct mst_mesh_desc {
  int n_nodes;
  const double *node_xy;  /* [n_nodes][2] */
  int n_cells;
  int n_faces;
  const int *face_nodes;  /* [n_faces][2], 0-based */
  const int *face_cells;  /* [n_faces][2], c1 = -1 on boundary faces */
  int n_zones;
  const int *zones;       /* [n_zones][4]: id, first face (1-based), last, type */
  /* Optional periodic images: [n_faces][2] translation that maps cell c1's
   * coordinates into the frame of the face (zero for ordinary faces); NULL
   * for none.  Periodic faces are interior faces (zone type 2). */
  const double *c1_shift;
} mst_mesh_desc;

/* Builds a mesh from raw arrays (same geometry rules as mst_mesh_read_msh);
 * replaces MshBlock::dataToMesh2D for generated meshes. */
mst_status mst_mesh_create(const mst_mesh_desc *desc, mst_mesh **out);
void mst_mesh_destroy(mst_mesh *m);

typedef struct mst_mesh_info {
  int n_nodes, n_cells, n_faces, n_int_faces, n_zones, n_cell_faces;
  int n_inner, n_bond1, n_bond2; /* MshBlock boundary lists (:370-406) */
  int n_tiles;                   /* device cell tiles */
  /* device layout: faces each tile borrows from another, halo entries over
   * all tiles, distinct halo cells and their cell-faces (what the FP32
   * flux kernel reads beyond its own cells when it forms the gradients) */
  int n_borrowed, n_halo, n_halo_cells, n_halo_cell_faces;
} mst_mesh_info;
mst_status mst_mesh_get_info(const mst_mesh *m, mst_mesh_info *info);

/* Exports the host geometry in file numbering, for parity checks; every
 * pointer may be NULL.  Sizes follow mst_mesh_info.  face_flag holds the
 * reference's flagLeftRight as 0/1 bytes [n_faces][2]. */
typedef struct mst_mesh_arrays {
  double *face_ctr, *face_dir, *face_area, *face_eta0; /* [nF][2],[nF][2],[nF],[nF] */
  int *face_dac;                                       /* [nF] */
  uint8_t *face_flag;                                  /* [nF][2] */
  int *face_cells;                                     /* [nF][2] */
  int *cell_ptr, *cell_faces, *cell_nb;                /* CSR, file order */
  double *cell_dof, *cell_eta0c;                       /* [tot][2], [tot] */
  double *cell_ctr, *cell_vol;                         /* [nC][2], [nC] */
  int *inner, *bond1, *bond2;
  int *cell_perm;   /* [nC] device slot of each file-numbered cell */
  int *face_perm;   /* [nF] device slot of each file-numbered face */
} mst_mesh_arrays;
mst_status mst_mesh_get_arrays(const mst_mesh *m, mst_mesh_arrays *a);

/* 3D meshes: MshBlock::readMsh with DIM 3 (mesh/MshBlock.cpp:436-789) --
 * triangular/quadrilateral faces, zones with a fixed face node count as the
 * reference reads them and, beyond it, mixed zones (node count 0 in the
 * zone header, each face line led by its node count).  Geometry by the
 * reference's 3D formulas (Face.cpp:20-39, Cell.cpp:6-14, :52-59; its cell
 * volume is the incomplete formula of the reference) plus the corrected
 * divergence-theorem volume.  mst_ctx3d_* below run the 3D residual path
 * on them. */
typedef struct mst_mesh3d mst_mesh3d;
typedef struct mst_mesh3d_info {
  int n_nodes, n_cells, n_faces, n_int_faces, n_zones, n_face_nodes, n_cell_faces,
      n_cell_nodes, n_inner, n_bond1, n_bond2;
} mst_mesh3d_info;
typedef struct mst_mesh3d_arrays {
  double *node_xyz;                                   /* [nN][3] */
  int *face_ptr, *face_nodes, *face_cells, *face_type; /* [nF+1], [..], [nF][2], [nF] */
  double *face_ctr, *face_dir, *face_area, *face_eta0; /* [nF][3], [nF][3], [nF], [nF] */
  double *face_cmd;     /* [nF][3] centre minus the mean of the two cell centres */
  int *face_dac;        /* [nF] */
  uint8_t *face_flag, *face_flag_set;  /* [nF][3] where set, [nF] */
  int *cell_ptr, *cell_faces, *cell_nb;               /* CSR, file order */
  double *cell_dof, *cell_eta0c;                      /* [tot][3], [tot] */
  double *cell_ctr, *cell_vol, *cell_vol_fixed;       /* [nC][3], [nC], [nC] */
  int *cell_node_ptr, *cell_nodes;                    /* reader's node order */
  int *inner, *bond1, *bond2, *cell_n_lower;
} mst_mesh3d_arrays;
mst_status mst_mesh3d_read_msh(const char *path, mst_mesh3d **out);
mst_status mst_mesh3d_get_info(const mst_mesh3d *m, mst_mesh3d_info *info);
/* Copies out the arrays; every pointer may be NULL. */
mst_status mst_mesh3d_get_arrays(const mst_mesh3d *m, mst_mesh3d_arrays *a);
void mst_mesh3d_destroy(mst_mesh3d *m);
/* A 3D mesh from arrays (generated meshes): face_ptr [nF+1] into
 * face_nodes (3 or 4 nodes per face), face_cells [nF][2] (c1 = -1 on
 * boundary faces), zones [n_zones][4] (id, first, last (1-based), Fluent
 * type); c1_shift (nullable) [nF][3] = x(c0's frame) - x(c1's frame) of
 * every face (non-zero on periodic faces, whose nodes are given in c0's
 * frame).  Holds the arrays only: the reference-geometry arrays of
 * mst_mesh3d_get_arrays stay empty for such a mesh. */
mst_status mst_mesh3d_from_arrays(int n_nodes, const double *node_xyz, int n_cells, int n_faces,
                                  const int *face_ptr, const int *face_nodes,
                                  const int *face_cells, int n_zones, const int *zones,
                                  const double *c1_shift, mst_mesh3d **out);

/* ------------------------------------------------------------------ */
/* 3D residual path                                                    */
/* ------------------------------------------------------------------ */
/* The reference's 3D path cannot run (2D-only thermodynamics,
 * work/FUNCTION.cpp:3-18; wrong 3D volume and quad area, Cell.cpp:52-59,
 * Face.cpp:30-36).  This is its 2D density path (RhoSolver.cpp:37-453, the
 * corrected mode of mst_ctx) carried to 3D: corrected geometry (face
 * centre = node mean, area 1/2 (n1-n0)x(n2-n0) or 1/2 (n2-n0)x(n3-n1),
 * cell centre = mean of face centres, divergence-theorem volume), Green-
 * Gauss gradient, split-axis Roe flux per axis (SolverRoe.cpp:70-123 with
 * |A| dQ in closed form), unlimited or limited MUSCL, the laminar viscous
 * term, BC zones as in 2D, explicit RK2 at a global CFL step.  States are
 * [n_cells][5] (rho, rho u, rho v, rho w, E) in file order. */
typedef struct mst_params3d {
  int precision;     /* MST_PREC_* */
  int order;         /* 1 or 2 */
  int limiter;       /* MST_LIMITER_* (order 2) */
  int viscous;       /* laminar viscous term (order 2) */
  double mu, lambda, kappa, cv;
  double inlet_q[5]; /* state of inlet faces */
  double cfl;        /* CFL number of the global step */
} mst_params3d;
void mst_params3d_default(mst_params3d *p);
typedef struct mst_ctx3d mst_ctx3d;
typedef struct mst_ctx3d_info {
  int n_cells, n_faces, n_tiles, max_tile_faces;
  int n_cell_faces;   /* CSR length */
  int n_borrowed;     /* faces listed by a second tile (cut by tile borders) */
  size_t device_bytes;
} mst_ctx3d_info;
mst_status mst_ctx3d_create(const mst_mesh3d *m, const mst_params3d *p, mst_ctx3d **out);
mst_status mst_ctx3d_destroy(mst_ctx3d *c);
mst_status mst_ctx3d_info_get(mst_ctx3d *c, mst_ctx3d_info *info);
mst_status mst_ctx3d_set_state(mst_ctx3d *c, const double *q);
mst_status mst_ctx3d_get_state(mst_ctx3d *c, double *q);
/* residual R [n_cells][5] of the current state (sum over the cell's faces,
 * ascending face id, of S_out . F); gradient [n_cells][3][5] */
mst_status mst_ctx3d_residual(mst_ctx3d *c, double *r);
mst_status mst_ctx3d_gradient(mst_ctx3d *c, double *g);
/* nsteps RK2 steps at the global CFL step, the state kept in HBM; t_end >
 * 0 cuts the last step to reach it.  Simulated time through *time
 * (nullable).  MST_EDIVERGED when a step before t_end had zero length
 * (some cell's CFL step was not positive: NaN or non-positive density or
 * pressure).  mst_ctx3d_last_timing: device milliseconds and kernel
 * launches of the last mst_ctx3d_step. */
mst_status mst_ctx3d_step(mst_ctx3d *c, int nsteps, double t_end, double *time);
mst_status mst_ctx3d_last_timing(mst_ctx3d *c, double *ms, int *launches);
/* sum over cells of 1/2 |rho u|^2 / rho V, and of V */
mst_status mst_ctx3d_kinetic_energy(mst_ctx3d *c, double *ke, double *vol);
/* Per-kernel CUDA-event timing of mst_ctx3d_step launches (as
 * mst_profile_*): on != 0 starts recording and clears the totals. */
mst_status mst_ctx3d_profile(mst_ctx3d *c, int on);
int mst_ctx3d_profile_count(mst_ctx3d *c);
mst_status mst_ctx3d_profile_get(mst_ctx3d *c, int i, char *name, size_t name_len, int *launches,
                                 double *total_ms);

/* ------------------------------------------------------------------ */
/* solver contexts: the RhoSolver surface                              */
/* ------------------------------------------------------------------ */
typedef struct mst_ctx mst_ctx;

/* RhoSolver(MshBlock*, fstream*, AllData*) (RhoSolver.h:17): uploads the
 * mesh once and allocates the device state.  The mesh must outlive it. */
mst_status mst_ctx_create(const mst_mesh *m, const mst_params *p,
                          mst_ctx **out);
mst_status mst_ctx_destroy(mst_ctx *c);
/* Replaces the parameters (the mesh stays resident). */
mst_status mst_ctx_set_params(mst_ctx *c, const mst_params *p);

/* RhoSolver::setDT (RhoSolver.cpp:33-35). */
mst_status mst_set_dt(mst_ctx *c, double dt);

/* Old state in (AllData p1OldCellQs, the Q that solve() reads). */
mst_status mst_set_state(mst_ctx *c, const double *q, size_t stride);
/* getOldValue (RhoSolver.cpp:504-506). */
mst_status mst_get_state(mst_ctx *c, double *q, size_t stride);
/* getNewValue (RhoSolver.cpp:507-509): the state solve() produced. */
mst_status mst_get_new_state(mst_ctx *c, double *q, size_t stride);

/* RhoSolver::solve (RhoSolver.cpp:37-89): one residual evaluation and one
 * explicit update Qnew = Qold - DT/V*R into the new-state buffer. */
mst_status mst_solve(mst_ctx *c);
/* RhoSolver::updateNewToOld (RhoSolver.cpp:513-517). */
mst_status mst_update_new_to_old(mst_ctx *c);

/* Per-cell residual R of the last mst_solve(), [n_cells][4] (the
 * reference's integralConvectFlux, RhoSolver.cpp:47-56).  mst_step does not
 * store it. */
mst_status mst_get_residual(mst_ctx *c, double *r, size_t stride);
/* Per-face flux matrices of the last solve(), [n_faces][2][4]
 * (p1OldFaceConvectFlux, RhoSolver.cpp:90-369). */
mst_status mst_get_face_flux(mst_ctx *c, double *f);
/* Cell gradients of the last 2nd-order solve(), [n_cells][2][4]
 * (p1NewCellGradFlux, RhoSolver.cpp:430-453). */
mst_status mst_get_gradient(mst_ctx *c, double *g);

/* Norms of one step. */
typedef struct mst_norms {
  double linf_change[4]; /* Time::goNextTimeStep, time/Time.cpp:69-76 */
  double l2_resid[4];    /* sqrt(sum_c (R_c/V_c)^2 / n_cells) */
  double dt;             /* step actually taken */
  double time;           /* simulated time after the step */
  double mass;           /* sum_c V_c * rho_c (conservation check) */
} mst_norms;

/* One residual evaluation and explicit update (what mst_solve does, with
 * the context's parameters and fixed dt) on device buffers the caller owns,
 * allocating nothing during the call.  No counterpart in the reference: it
 * serves programs that embed the solver in a GPU application which manages
 * all device memory itself and forbids cudaMalloc/cudaFree while running
 * (cudaFree synchronises the whole device; a pool may have no room), and
 * loops that must avoid those implicit synchronisations.  The context is
 * created once at set-up (that call does allocate).
 * The context must use one Euler stage at a fixed dt (MST_TIME_EULER,
 * MST_DT_FIXED; others: MST_EUNSUPPORTED); any precision, order, limiter
 * and viscous setting.
 *   q_dev, qnew_dev  [n_cells][4] doubles in the context's device cell order
 *                    (mst_mesh_arrays.cell_perm gives each file cell's row),
 *                    32-byte aligned; q_dev is read, qnew_dev written; the
 *                    buffers (r_dev included) must not overlap (MST_EINVAL)
 *   r_dev            optional [n_cells][4] residual output (same order)
 *   norms_dev        optional 10 doubles: linf_change[4], l2_resid[4],
 *                    mass, dt
 * Scratch (gradients, norm partials) is one fixed file-scope device array of
 * about 8.1 MiB that every GPU loading the library keeps until exit, so the
 * mesh may have at most 131072 cells (larger meshes: MST_EINVAL).  All calls
 * share that array: calls that overlap on the GPU race and must be
 * serialised by the caller.  Every call looks up the array's device
 * address on the current device; the first call on a device is the set-up
 * (it may load the library's device code), so make it before any stream
 * capture. 
 * Runs on the context's stream and returns when the outputs are written;
 * the caller must have finished writing q_dev before the call.  On the FP32
 * path the update is done in FP64 on the caller's buffers (mst_solve keeps
 * that path's state as float pairs), so the two agree to FP32 rounding. */
mst_status mst_solve_device_noalloc(mst_ctx *c, const double *q_dev,
                                   double *qnew_dev, double *r_dev,
                                   double *norms_dev);

/* Device-resident time stepping: nsteps steps of the configured scheme
 * without host round trips (the Work::work loop, work/Work.cpp:53-89, with
 * the state kept in HBM).  t_end > 0 clips the last step to reach t_end
 * exactly.  last (nullable) receives the norms of the final step.
 * Returns MST_EDIVERGED when the final step's residual or mass is not
 * finite (the state left the physical range). */
mst_status mst_step(mst_ctx *c, int nsteps, double t_end, mst_norms *last);

/* Host-held states stepped through the device with the copies hidden
 * behind the computation (the reference's time loop keeps its state on the
 * host and hands it to the solver every step, Time.cpp:54-80): job j
 * copies q_in[j] ([n_cells][4] doubles, file order) to the device, takes
 * nsteps steps of the configured scheme from it, and copies the result to
 * q_out[j].  The copy-in of job j+1 and the copy-out of job j-1 run on
 * their own streams while job j computes (two staging slots each way,
 * allocated on the first call).  Use page-locked host buffers
 * (mst_host_alloc) for full-speed copies.  Returns when every q_out is
 * written; the context's state is then the last job's result.
 * MST_EDIVERGED when a job's last-step residual or mass is not finite. */
mst_status mst_step_host_jobs(mst_ctx *c, int n_jobs, const double *const *q_in,
                              double *const *q_out, int nsteps);

/* Simulated time of the context (sum of the steps taken). */
mst_status mst_get_time(mst_ctx *c, double *t);

/* Launch-level timing of the most recent mst_step/mst_solve on the
 * context's stream: elapsed milliseconds between its first and last
 * kernel, and the number of kernels launched. */
mst_status mst_last_timing(mst_ctx *c, double *ms, int *launches);

/* ------------------------------------------------------------------ */
/* batched steady solves (implicit LU-SGS)                             */
/* ------------------------------------------------------------------ */
/* No counterpart in the reference, whose density-based path is explicit
 * only: many independent cases, each a mesh with its own inflow state and
 * transport coefficients, iterated together on one GPU to a residual
 * tolerance by matrix-free LU-SGS (Yoon-Jameson: scalar diagonal from the
 * spectral radii, Euler-flux differences off the diagonal), with local
 * steps from a per-case CFL number that grows as the residual falls
 * (switched evolution relaxation), and Gauss-Seidel sweeps over colour
 * groups of the cell adjacency (one launch per colour and direction).
 * The residual is the corrected-mode (reference_quirks = 0) residual of
 * mst_params, in its precision; the sweeps and the state are FP64. */
typedef struct mst_batch mst_batch;

typedef struct mst_case_params {
  double inlet_q[4];               /* type-10 boundary state of the case */
  double mu, lambda, kappa, cv;    /* transport coefficients (viscous runs) */
} mst_case_params;

typedef struct mst_implicit_params {
  double cfl0;      /* CFL of the first iteration */
  double cfl_max;   /* ceiling of CFL = cfl0 * L2_first / L2 */
  double omega;     /* LU-SGS relaxation of the spectral radii (>= 1) */
  double tol;       /* a case has converged when L2 <= tol * L2_first; its
                     * state is kept from then on */
  /* limiter freezing (default 0.1): once a case is below freeze_tol *
   * L2_first and its L2 fell by less than 30% over the last 50
   * iterations, the next iteration records the ratio slope / (upwind
   * difference) of every limited face side; later iterations reconstruct
   * with those ratios times the current upwind differences, so the
   * limiter's switching no longer stalls convergence (0: never).  Every update is halved (at most 6 times, else
   * dropped) until density and pressure stay above a fifth of their
   * current values. */
  double freeze_tol;
  /* mixed precision (FP64 production path only): every case starts with
   * the FP32 residual (FP32 gradient, reconstruction and flux; FP64 sweeps
   * and state) and switches, on its own, to the FP64 residual once it is
   * below fp32_until * L2_first or stagnating in FP32 (its L2 has not
   * fallen by 10% for fp32_window iterations: the FP32 residual's floor);
   * cases in the two phases iterate side by side (one residual pass per
   * phase, each skipping the other phase's cases); 0: FP64 residual
   * throughout */
  double fp32_until;
  int max_iter;     /* iteration limit of mst_batch_solve */
  int graph_iters;  /* iterations per CUDA-graph launch (even; 0: no graph) */
  int autotune;     /* time the sweep block sizes once and keep the fastest */
  /* FP32 sweeps (production paths): the off-diagonal flux differences and
   * spectral radii in FP32 on FP32 copies of the state and of dQ; the
   * diagonal, its inversion and the state update stay FP64.  The residual
   * that decides convergence is unchanged, so the converged state meets
   * the same tolerance. */
  int sweep_fp32;
  /* temperature floor (0: off): an updated state with p < p_floor * rho
   * gets its internal energy raised to p = p_floor * rho (density and
   * momentum kept).  Without it a near-vacuum cell at a slip / no-slip
   * corner rejects every update (positivity) and freezes its case. */
  double p_floor;
  /* iterations of the FP32-phase stagnation test; 0 = 500 */
  int fp32_window;
  /* re-freezing (default 500; 0: off): a case whose frozen-limiter L2 has
   * not fallen below 0.9 of its best for refreeze_window iterations records
   * the limiter ratios again from its current state (a limiter frozen on
   * a field still far from the solution can hold a case at a plateau) */
  int refreeze_window;
  /* stall retirement (0: off): a case whose L2 has not fallen below half
   * of its best for stall_window iterations of its FP64 phase is retired
   * (MST_CASE_STALLED) and costs nothing afterwards; if fallback states
   * are set (mst_batch_set_fallback) it is restarted from its fallback
   * state instead, once per solve from a set state */
  int stall_window;
  /* with fallback states set: a case not converged restart_after
   * iterations after the state was set restarts from its fallback state,
   * once (0: off) -- a fixed budget; it also restarts cases that are slow
   * but would converge, which restart_projected leaves alone */
  int restart_after;
  /* with fallback states set: every restart_projected iterations after
   * the state was set, a case whose L2, extrapolated at its rate over the
   * last window, would not reach the tolerance within max_iter -- in two
   * windows in a row, counted in its FP64 phase -- restarts from its
   * fallback state, once (0: off): a slow warm start gives way to the
   * free stream while a slow case that will still make the cap is left
   * alone */
  int restart_projected;
} mst_implicit_params;

/* cfl0 50, cfl_max 100, omega 1.2, tol 1e-8, freeze_tol 1e-1,
 * fp32_until 0, max_iter 20000, graph_iters 20, autotune on,
 * sweep_fp32 off, p_floor 0, refreeze_window 500, stall_window 0,
 * restart_after 0, restart_projected 0. */
void mst_implicit_params_default(mst_implicit_params *p);

typedef struct mst_batch_info_t {
  int n_cases, n_cells, n_faces, n_colors, sweep_threads, graph_iters;
} mst_batch_info_t;

typedef struct mst_batch_result {
  int iterations;        /* iterations run by this call */
  int total_iterations;  /* since the state was set */
  int n_converged;       /* cases at tolerance */
  double ms;             /* device time of the call */
  int n_diverged;        /* cases retired as diverged (MST_CASE_DIVERGED) */
  int n_stalled;         /* cases retired as stalled (MST_CASE_STALLED) */
  int n_restarted;       /* cases restarted from their fallback states */
} mst_batch_result;

/* Joins the meshes into one device mesh (cases keep their cells together)
 * and allocates the batch.  L2 = sqrt(mean over the case's cells of
 * (R_rho / V)^2), normalised by its value at the first iteration. */
mst_status mst_batch_create(const mst_mesh *const *meshes,
                            const mst_case_params *cases, int n_cases,
                            const mst_params *p, const mst_implicit_params *ip,
                            mst_batch **out);
mst_status mst_batch_destroy(mst_batch *b);
mst_status mst_batch_info(const mst_batch *b, mst_batch_info_t *info);
/* Colour of every cell, cases in order, file numbering within a case. */
mst_status mst_batch_colors(const mst_batch *b, int *color);
/* States of all cases, cases in order, rows of 4 doubles; setting the
 * state restarts the convergence bookkeeping. */
mst_status mst_batch_set_state(mst_batch *b, const double *q);
/* Reference L2 per case [n_cases] (after mst_batch_set_state, which clears
 * it): the tolerance, the SER CFL and limiter freezing then measure L2
 * against it instead of the first iteration's L2 -- e.g. a warm-started
 * solve held to the same absolute residual as the cold start it is
 * compared with.  NULL clears it. */
mst_status mst_batch_set_l2_ref(mst_batch *b, const double *l2_ref);
mst_status mst_batch_get_state(mst_batch *b, double *q);
/* Exactly n iterations (no convergence stop, no graph). */
mst_status mst_batch_iterate(mst_batch *b, int n);
/* Iterates until every case has converged or max_iter iterations ran. */
mst_status mst_batch_solve(mst_batch *b, mst_batch_result *res);
/* Per case: the iteration at which it converged (-1: not yet;
 * MST_CASE_DIVERGED: retired because its L2 stopped being finite, which a
 * non-positive density or pressure causes through the sound speed;
 * MST_CASE_STALLED: retired by the stall_window test; a retired case's
 * cells cost nothing from the next iteration on and the other cases run
 * on), the first and the latest L2 (each nullable). */
enum { MST_CASE_DIVERGED = -2, MST_CASE_STALLED = -3 };
mst_status mst_batch_case_status(mst_batch *b, int *conv_iter,
                                 double *first_l2, double *last_l2);
/* Fallback states of all cases (the layout of mst_batch_set_state; NULL
 * clears them), e.g. the free stream behind a learned initial field.  A
 * case restarted from its fallback state iterates exactly as a solve
 * started from that state would -- its CFL ramp, limiter freezing,
 * precision phase and stall test start over; the reference L2 of a
 * restarted case is its first L2 after the restart unless
 * mst_batch_set_l2_ref fixed it -- with its iteration numbers shifted by
 * the iteration of the restart. */
mst_status mst_batch_set_fallback(mst_batch *b, const double *q);
/* Restarts the listed cases (indices, each once in the list) from their
 * fallback states at the current iteration, whatever their status;
 * MST_EINVAL without fallback states. */
mst_status mst_batch_restart(mst_batch *b, const int *cases, int n);
/* Per case the iteration of its latest restart since the state was set,
 * -1 if none. */
mst_status mst_batch_case_restarts(mst_batch *b, int *restart_iter);

/* ------------------------------------------------------------------ */
/* tensor-core GEMM of the learned initial field                       */
/* ------------------------------------------------------------------ */
/* No counterpart in the reference.  Check entry point of the BF16
 * tensor-core GEMM (tcgen05, accumulator in tensor memory) used by the
 * network's dense layers: C[M][N] = A[M][K] . B[N][K]^T (+ bias[N]) (ReLU),
 * A and B BF16 bit patterns (row-major), C FP32 (row-major), K a multiple
 * of 64.  Host buffers; copies in and out.  layout 0 is the production
 * descriptor layout; 1 swaps its two strides (a check of the layout); a
 * multiple of 64 splits K into chunks of that size over separate CTAs
 * whose partial products are added in a fixed order (no bias / ReLU). */
mst_status mst_tc_gemm_check(const uint16_t *A, const uint16_t *B,
                             const float *bias, float *C, int M, int N, int K,
                             int relu, int layout);

/* No counterpart in the reference.  Every device-side wait of the
 * library's kernels (the tensor-core GEMM's mbarrier waits) is bounded:
 * after `polls` polls it gives up, the kernel finishes its own in-flight
 * work, frees what it holds and returns, and the call reports
 * MST_ETIMEOUT; the context stays usable.  polls < 0 restores the default
 * (2^26); 0 makes every such wait give up at once, which tests the timeout
 * path without a hang.  Process-wide. */
mst_status mst_set_wait_limit(long long polls);

/* ------------------------------------------------------------------ */
/* learned initial field                                                */
/* ------------------------------------------------------------------ */
/* No counterpart in the reference.  A message-passing network over the
 * cell adjacency predicts a steady field from cell geometry and the flow
 * parameters, to start the batched implicit solves from:
 *   h0 = relu(We x + be),  x = 16 features per cell
 *   h_{l+1} = h_l + relu(Wl [h_l, mean of the neighbours' h_l] + bl),
 *             l = 0, 1, 2, width 128
 *   y = Wd h3 + bd,  4 outputs per cell
 * Dense layers run on the tensor cores (BF16 operands, FP32 accumulation,
 * both forward and backward); master weights and Adam moments FP32.
 * Parameters, in order: We [128][64] (columns >= 16 unused), be [128],
 * then per layer Wl [128][256], bl [128], then Wd [4][128], bd [4];
 * row-major [outputs][inputs]. */
typedef struct mst_mpnn mst_mpnn;
int mst_mpnn_num_params(void);
/* Glorot-uniform weights from a seeded generator, zero biases. */
mst_status mst_mpnn_create(uint64_t seed, mst_mpnn **out);
mst_status mst_mpnn_destroy(mst_mpnn *m);
/* The graph the next forward/backward run on: features [n][16], CSR
 * neighbour lists (nbr_ptr [n+1], nbr ids in [0, n)). */
mst_status mst_mpnn_set_graph(mst_mpnn *m, int n, const float *features,
                              const int *nbr_ptr, const int *nbr);
/* Targets [n][4] of the mean-squared-error loss. */
mst_status mst_mpnn_set_targets(mst_mpnn *m, const float *t);
/* Outputs [n][4] (y nullable). */
mst_status mst_mpnn_forward(mst_mpnn *m, float *y);
/* Gradients of the loss of the last forward; loss nullable. */
mst_status mst_mpnn_backward(mst_mpnn *m, double *loss);
/* which = 0: parameters, 1: gradients; out [mst_mpnn_num_params()]. */
mst_status mst_mpnn_get(mst_mpnn *m, int which, float *out);
mst_status mst_mpnn_set_weights(mst_mpnn *m, const float *w);
/* One Adam step (beta 0.9 / 0.999) with the current gradients. */
mst_status mst_mpnn_adam_step(mst_mpnn *m, float lr);
/* Live timing of the network's tensor-core GEMM launches: on != 0 starts
 * recording (a CUDA event pair around every GEMM launch), 0 stops; both
 * clear what was recorded.  profile_read synchronises the device and
 * returns out[0] = summed GEMM milliseconds, out[1] = their 2MNK flops,
 * out[2] = their operand and result bytes, out[3] = launches, then clears
 * the record.  No reference counterpart (the reference has no network). */
mst_status mst_mpnn_profile(mst_mpnn *m, int on);
mst_status mst_mpnn_profile_read(mst_mpnn *m, double out[4]);

/* ------------------------------------------------------------------ */
/* result writer and checkpoint files                                  */
/* ------------------------------------------------------------------ */
/* Node averages of the current state, computed on the device as
 * Work::writedataRhoBasedMshNodePlt does (work/Work.cpp:240-300): face
 * values (eta0 blend on type-2 faces, the cell value on boundary faces),
 * averaged onto each node over its faces with weights 1/area.  With
 * reference_quirks the weight of every face of node i is 1/area of face i
 * (Work.cpp:292-293 index faces by the node id; the call then needs
 * n_nodes <= n_faces); without, each face's own 1/area.
 * node_q [n_nodes][4] conserved, node_vars [n_nodes][6] = rho, u, v, T, p,
 * Ma (work/FUNCTION.cpp:8-20, cv from the parameters); nodes in file
 * order; either may be NULL. */
mst_status mst_node_values(mst_ctx *c, double *node_q, double *node_vars);

/* Tecplot ASCII file of the current state: the format of
 * Work::writedataRhoBasedMshNodePlt (Work.cpp:204-319), zone title zone_t,
 * one POINT row X Y rho u v T p Ma per node ("%.15f", space-terminated),
 * then 1-based node lists per cell in the reader's node order
 * (mesh/MshBlock.cpp:335-367).  With reference_quirks the file is
 * byte-identical to the reference's (its stray title quote, zone type
 * FEQUADRILATERAL for every mesh, 3 ids for triangles, quads in the
 * reader's node order, which is a bow tie); without, the title is well
 * formed, all-triangle meshes are FETRIANGLE zones, quads are written in
 * cyclic order (0 1 3 2 of the reader's) and triangles in mixed zones
 * repeat their last node. */
mst_status mst_write_plt(mst_ctx *c, const char *path, int zone_t);

/* Text checkpoint of the current state: one line per cell (file order) of
 * 4 "%.15f" numbers, each followed by a space, the format of
 * Work::writedataCellContinue (Work.cpp:483-514).  Not exact: 15
 * decimals. */
mst_status mst_write_cell_text(mst_ctx *c, const char *path);
/* Reads such a file into the state, as Work::readPbasedCellPlt
 * (Work.cpp:432-482) does: the first 4 space-separated numbers of each
 * line.  MST_EINVAL (and the state unchanged) on a missing file, too few
 * lines or too few numbers on a line. */
mst_status mst_read_cell_text(mst_ctx *c, const char *path);

/* Exact binary checkpoint: the FP64 state, on the FP32 path also the
 * float-pair parts, the time and the last step length, behind an 88-byte
 * header carrying a hash of the mesh (node coordinates, face nodes, face
 * cells, face types) and FNV-1a 64 checksums of header and payload.  Load
 * rejects (MST_EINVAL, state unchanged) files of another mesh, truncated
 * or corrupted files.  Restarting from a checkpoint continues bit-for-bit
 * like the uninterrupted run. */
mst_status mst_checkpoint_save(mst_ctx *c, const char *path);
mst_status mst_checkpoint_load(mst_ctx *c, const char *path);

/* ------------------------------------------------------------------ */
/* sparse LU-SGS / Gauss-Seidel sweeps (the reference's lusolver)      */
/* ------------------------------------------------------------------ */
typedef struct mst_lu mst_lu;
enum { MST_LU_ILUSGS = 0, MST_LU_GS = 1 };

/* A sparse system given as the ordered insertions the reference's solvers
 * receive: block = 1 replaces SparseSolverNUM built with setELE (ops[i] =
 * 0) / addELE (ops[i] = 1) (lusolver/SparseSolverNUM.cpp:115-140); block =
 * 4 replaces SparseSolver<Matrix4d, Vector4d> built with setD/setL/setU
 * (lusolver/SparseSolver.cpp:35-48), vals then holding row-major 4x4 blocks
 * (ops may be NULL).  Duplicates are kept, as in the reference.  Rows are
 * grouped into dependency levels for the GPU sweeps. */
mst_status mst_lu_create(int block, int dim, int n, const int *rows,
                         const int *cols, const int *ops, const double *vals,
                         mst_lu **out);
/* SparseSolverNUM::solveILUSGS (SparseSolverNUM.cpp:144-212) or solveGS
 * (:214-252) for block = 1; SparseSolver::solveILU (SparseSolver.cpp:53-104)
 * for block = 4.  x holds the initial guess and receives the solution;
 * iterations (nullable) receives the outer iterations run (at most
 * LU_INTERVAL = 5, fewer when the reference's exit test triggers).  Results
 * are bit-identical to the reference's. */
mst_status mst_lu_solve(mst_lu *s, int method, const double *b, double *x,
                        int *iterations);
/* Number of dependency levels of the forward and backward sweeps. */
mst_status mst_lu_levels(const mst_lu *s, int *forward, int *backward);
mst_status mst_lu_destroy(mst_lu *s);

/* ------------------------------------------------------------------ */
/* pressure-based SIMPLE solver (the reference's PSolver/SolverSIMPLE) */
/* ------------------------------------------------------------------ */
/* Replaces PSolver (pSolver/PSolver.h:16-41) with PSOLVER = SolverSIMPLE
 * (pSolver/SolverSIMPLE.h:20-80), the solver the reference's CONST.h
 * selects (RHO_P 1).  States are (p, u, v, T) per cell ([n_cells][4], file
 * cell order, as AllData's pNewCellPUVT) and per face ([n_faces][4], as
 * pFacePUVTSC).  Results are bit-identical to the reference's SolverSIMPLE
 * (one OpenMP thread; the reference's residual maximum races across
 * threads, its state does not). */
typedef struct mst_simple mst_simple;
typedef struct mst_simple_params {
  double dt;          /* PSolver::setDT (reference: 1 / STEP_TIME) */
  double alpha_p;     /* SIMPLE_ALPHA_P: p += alpha_p p' */
  int n_inner;        /* SIMPLE_INTERVAL: SIMPLE iterations per step */
  int wall_smooth;    /* FLAG_WALLSMOOTH: 1 reflects the wall velocity,
                         0 sets it to zero (SolverSIMPLE.cpp:131-138) */
  double inlet[4];    /* face (p, u, v, T) of inlet (type 10) faces */
  double p_out;       /* face pressure of outlet (type 5) faces */
  int cluster;        /* CTAs of the kernel's thread-block cluster, 0 = the
                         largest that fits (16, 8, 4, 2 or 1) */
  int reserved[3];
} mst_simple_params;
typedef struct mst_simple_info {
  int n_cells, n_faces;
  int cluster, threads;               /* launch shape of the step kernel */
  int momentum_levels, pressure_levels; /* Gauss-Seidel sweep levels */
  int last_steps;                     /* steps of the last mst_simple_step */
  int batch_cluster;                  /* CTAs per cluster of the last
                                         mst_simple_step_batch led by it */
} mst_simple_info;

/* The reference's CONST.h values: dt = 1/4000, alpha_p = 0.3, n_inner = 5,
 * wall_smooth = 1, inlet = (getP(inletQ), 0, 0, inletT) and p_out =
 * getP(iniQ) (SolverSIMPLE.cpp:110-112, :168-175). */
mst_status mst_simple_default_params(mst_simple_params *p);
/* (p, u, v, T) of conserved states (rho, rho u, rho v, E) as
 * Time::initialization forms them (time/Time.cpp:21-23; getP/getT,
 * work/FUNCTION.cpp:7-14).  Host only. */
mst_status mst_q_to_puvt(int n, const double *q, double *puvt);
/* params may be NULL (defaults).  Periodic meshes: MST_EUNSUPPORTED. */
mst_status mst_simple_create(const mst_mesh *m, const mst_simple_params *p,
                             mst_simple **out);
/* Host arrays.  The old time level is set to the same state
 * (Time::initialization).  face_puvt may be NULL: face values are kept
 * (zero after create); faces of zone types the reference's face update
 * skips (e.g. 7) keep their values for the whole run. */
mst_status mst_simple_set_state(mst_simple *s, const double *cell_puvt,
                                const double *face_puvt);
mst_status mst_simple_get_state(mst_simple *s, double *cell_puvt, double *face_puvt);
/* nsteps time steps, each Time::goNextTimeStep with RHO_P 1 (time/Time.cpp:
 * 54-80): a SolverSIMPLE solve of n_inner iterations, then new -> old.
 * time_rows (nullable) receives [nsteps][4] max |new - old| / old per
 * component (the Time loop's log row).  One kernel launch. */
mst_status mst_simple_step(mst_simple *s, int nsteps, double *time_rows);
/* nsteps time steps of n independent cases in ONE launch, one
 * thread-block cluster per case, so that several cases fill the GPU; the
 * cluster size is chosen for the batch (as many cases resident at once as
 * pays off; results do not depend on it) and each case's results are those
 * of mst_simple_step.  time_rows (nullable): [n][nsteps][4]. */
mst_status mst_simple_step_batch(mst_simple *const *cases, int n, int nsteps,
                                 double *time_rows);
/* Of the last mst_simple_step: the SIMPLE iteration rows
 * [nsteps][n_inner][4] (max |new - old| / (old + EOR), SolverSIMPLE.cpp:
 * 62-71) and the Gauss-Seidel iterations of the u, v and p' solves
 * [nsteps][n_inner][3] (each at most LU_INTERVAL).  Either may be NULL. */
mst_status mst_simple_rows(mst_simple *s, double *inner_rows, int *gs_iters);
mst_status mst_simple_get_info(const mst_simple *s, mst_simple_info *info);
mst_status mst_simple_destroy(mst_simple *s);

/* Per-kernel CUDA-event timing on the context's stream.  When enabled,
 * every kernel launch of mst_solve/mst_step is bracketed by events; the
 * totals accumulate until mst_profile_reset. */
mst_status mst_profile_enable(mst_ctx *c, int on);
mst_status mst_profile_reset(mst_ctx *c);
/* Number of distinct kernels timed so far. */
int mst_profile_count(mst_ctx *c);
/* Stats of kernel i: its name (copied into name, NUL-terminated), number
 * of launches and total device milliseconds. */
mst_status mst_profile_get(mst_ctx *c, int i, char *name, size_t name_len,
                           int *launches, double *total_ms);

/* Page-locked host buffers for fast host<->device copies of states
 * (cudaHostAlloc / cudaFreeHost). */
mst_status mst_host_alloc(size_t bytes, void **out);
mst_status mst_host_free(void *p);

/* Number of CUDA devices visible to this process. */
mst_status mst_device_count(int *n);
/* Selects the device later contexts of this host thread are created on. */
mst_status mst_set_device(int device);

/* Measurement helper, no counterpart in the reference: the current
 * device's rate of FP64 fused multiply-adds (thread instructions per
 * second; 2 flops each), from a kernel of independent DFMA chains timed
 * with CUDA events.  The roof of the FP64-pipe-bound kernels. */
mst_status mst_probe_fp64_rate(double *dfma_per_s);

/* Text of the last error on this thread (static storage). */
const char *mst_last_error(void);
/* ABI version. */
int mst_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
