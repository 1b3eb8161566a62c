/* Implicit steady iterations of the oracle (TEST INFRASTRUCTURE ONLY; see
 * mstoracle.h and mstoracle_implicit.c). */
#ifndef MSTORACLE_IMPLICIT_H
#define MSTORACLE_IMPLICIT_H
#include "mstoracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct om_lusgs_params {
  double cfl0, cfl_max, omega;
  /* limiter freezing: the iteration after L2 first falls to freeze_tol *
   * L2_first records the limiter ratios slope / (upwind difference) of
   * every face, later iterations reuse them (0: never) */
  double freeze_tol;
  /* convergence: from the first iteration with L2 <= tol * L2_first on,
   * the state is kept (0: never) */
  double tol;
  /* temperature floor: an updated state with p < p_floor * rho gets its
   * internal energy raised to p = p_floor * rho (0: off) */
  double p_floor;
  /* re-freezing: a frozen case whose L2 has not fallen below 0.9 of its
   * best for refreeze_window iterations records the ratios again (0: off) */
  int refreeze_window;
} om_lusgs_params;

/* niter LU-SGS iterations of one case in place (corrected-mode residual of
 * p, which must have quirks = 0); color [n_cells] the colour of each cell;
 * l2_hist [niter] (nullable) the L2 of R_rho / V before each update (after
 * convergence nothing runs again and the converged L2 is repeated). */
int om_lusgs_iterate(const om_mesh *m, const om_params_ext *p, double *q,
                     const int *color, const om_lusgs_params *ip, int niter,
                     double *l2_hist);
/* Greedy colouring of the cell adjacency in file order; returns the count. */
int om_greedy_colors(const om_mesh *m, int *color);

#ifdef __cplusplus
}
#endif
#endif
