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

/* Case set-up of the oracle itself (lfm_port_setup.c): the solver description
 * of an in-memory polyMesh with its parameters and initial fields, built
 * without the device library. Whole cases in the reference's cell order only
 * (params->renumber must be LFM_RENUMBER_NONE). Returns 0 on success, -1 with
 * lfm_port_last_error() set otherwise. */
typedef struct lfm_port_case lfm_port_case;
int lfm_port_case_build(const lfm_polymesh* mesh, const lfm_params* params, const lfm_fields* fields,
                        lfm_port_case** out);
/* Pointers into the case's arrays, valid until lfm_port_case_free. */
int lfm_port_case_describe(const lfm_port_case* c, lfm_solver_desc* out);
/* polyMesh cell label of each solver-order cell ([n_cells]). */
int lfm_port_case_cell_ids(const lfm_port_case* c, int64_t* out);
void lfm_port_case_free(lfm_port_case* c);
const char* lfm_port_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
