/* CPU restatement of the reference time step (oracle). Test infrastructure
 * only: tests, the smoke check and the CPU baseline of bench.py call it; the
 * product path never does. */
#ifndef LFM_PORT_H
#define LFM_PORT_H

#include "lfm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Advances q ([nq][n_cells], solver order) by nsteps time steps of size dt.
 * residual (optional, [nq]) receives the last step's summed squared residual
 * when desc->residuals is set. Returns 0 on success. */
int lfm_port_run(const lfm_solver_desc* desc, double* q, int nsteps, double dt, double* residual);
/* As lfm_port_run; cell_res ([nq][n_cells]) receives the per-cell stage-0
 * residual (the reference's RES) of the last step when desc->residuals is set. */
int lfm_port_run_cell_residual(const lfm_solver_desc* desc, double* q, int nsteps, double dt, double* cell_res);
/* compute_cfl / compute_dt of the reference for state q. */
int lfm_port_cfl(const lfm_solver_desc* desc, const double* q, double dt, double* cfl);
int lfm_port_min_dt(const lfm_solver_desc* desc, const double* q, double max_co, double* dt);

#ifdef __cplusplus
}
#endif
#endif
