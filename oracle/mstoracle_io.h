/* Result writer and text checkpoint of the oracle (TEST INFRASTRUCTURE
 * ONLY; see mstoracle.h and mstoracle_io.c). */
#ifndef MSTORACLE_IO_H
#define MSTORACLE_IO_H
#include "mstoracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Node averages (Work.cpp:244-295): node_q [n_nodes][4], node_vars
 * [n_nodes][6] = rho u v T p Ma; either may be NULL. */
int om_node_values(const om_mesh *m, const double *q, int quirks, double cv,
                   double *node_q, double *node_vars);
/* Cell node lists of the reader (MshBlock.cpp:335-367). */
void om_cell_nodes(const om_mesh *m, int *ptr, int *ids);
/* Reference-format Tecplot file (Work.cpp:204-319). */
int om_write_plt(const om_mesh *m, const double *q, double cv, int zone_t,
                 const char *path);
/* Reference-format text checkpoint (Work.cpp:483-514). */
int om_write_cell_text(int n_cells, const double *q, const char *path);

#ifdef __cplusplus
}
#endif
#endif
