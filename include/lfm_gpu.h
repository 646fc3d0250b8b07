/* lfm_gpu.h - C ABI of the GB300 explicit finite-volume time step.
 *
 * This is the drop-in boundary for libFastMesh's hot path: the ISolver stage
 * methods driven by Mesh::solve (reference src/mesh_solver.cpp:474-727) and
 * the case input behind IMeshReader / CInputReader. Plain C types only: every
 * function returns 0 on success and a negative lfm_status on failure (the
 * message is available from lfm_last_error()); no C++ exception crosses it.
 * Handles are owned by the caller and must be released with the matching
 * *_free / *_destroy call. Calls on one solver handle are not re-entrant; one
 * solver issues all its work on its own CUDA stream.
 *
 * Arrays are structure-of-arrays: a field with k components over n entries is
 * k consecutive blocks of n values. Conserved state q = (rho, rho*u[dim],
 * rho*E), nq = dim + 2 components, cells in solver order (submesh 0 cells in
 * polyMesh order, then submesh 1 cells), exactly the order of the reference's
 * (submesh, index) numbering. */
#ifndef LFM_GPU_H
#define LFM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lfm_status {
    LFM_OK = 0,
    LFM_ERR_INVALID = -1,   /* bad argument or case data */
    LFM_ERR_IO = -2,        /* case files missing or malformed */
    LFM_ERR_CUDA = -3,      /* CUDA runtime error */
    LFM_ERR_NOMEM = -4,     /* device memory exhausted */
    LFM_ERR_NUMERIC = -5,   /* non-finite state detected */
    LFM_ERR_UNSUPPORTED = -6
} lfm_status;

/* Scheme ids, as the reference's fastmesh_solver_t (api/fastmesh.h:38-41). */
#define LFM_SOLVER_M1 0
#define LFM_SOLVER_M2 1
#define LFM_SOLVER_M2AUSM 2

/* Arithmetic of the flux kernels. LFM_FP64 is the plain method; LFM_FP32_BULK
 * computes fluxes, limiter and residual in FP32 and keeps the RK registers,
 * geometry precompute and dt reduction in FP64. */
#define LFM_FP64 0
#define LFM_FP32_BULK 1

/* Boundary-ghost kinds (reference src/cfd_v0.cpp:972-1005). */
#define LFM_GHOST_NONE 0
#define LFM_GHOST_WALL 1
#define LFM_GHOST_INLET 2
#define LFM_GHOST_OUTLET 3
#define LFM_GHOST_FARFIELD 4

/* Solver description: the reference's per-cell CFDv0_cell data after
 * CFDv0_solver::initialize + reorder_faces (src/cfd_v0.cpp:83-339, 759-967),
 * flattened. Faces are the "owned" cell-faces in the reference's processing
 * order (cell by cell, slot by slot); P is the processing cell, N the other
 * side (N >= n_cells: boundary ghost N - n_cells, then processor-face halo
 * N - n_cells - n_ghosts). Geometry is seen from P. */
typedef struct lfm_solver_desc {
    int dim;                 /* 2 or 3 */
    int nq;                  /* dim + 2 */
    int solver;              /* LFM_SOLVER_* */
    int rk_order;            /* stages per time step, 0..8 (0: a time step runs no stage) */
    int minmod;              /* fvSchemes lfm/minmodExists */
    int residuals;           /* controlDict lfm/post/haveResiduals */
    int64_t n_cells, n_cells0, n_ghosts, n_faces;
    const int64_t* face_p;   /* [n_faces] */
    const int64_t* face_n;   /* [n_faces] */
    const uint8_t* face_ghost; /* [n_faces] neighbour is a boundary ghost */
    const double* S;         /* [dim][n_faces] face area vector, outward from P */
    const double* d;         /* [dim][n_faces] P-centre to N-centre vector */
    const double* w;         /* [n_faces] linear weight of P */
    const double* smag;      /* [n_faces] |S| */
    const double* dmag_inv;  /* [n_faces] 1/|d| */
    const double* dnorm;     /* [dim][n_faces] d/|d| */
    const double* delta_mag; /* [n_faces] |delta|, delta = d |S|^2/(S.d) */
    const double* K;         /* [dim][n_faces] S - delta */
    const double* vol_inv;   /* [n_cells] */
    const double* sponge;    /* [n_cells] sponge sigma */
    const int64_t* ghost_cell; /* [n_ghosts] interior cell of each ghost */
    const int* ghost_kind;   /* [n_ghosts] LFM_GHOST_* */
    const int64_t* cell_face_offsets; /* [n_cells+1] incidence, ascending face */
    const int64_t* cell_faces;
    const int8_t* cell_face_sign;     /* +1 when the cell is P */
    const int64_t* cell_s_offsets;    /* [n_cells+1] all valid faces of a cell */
    const double* cell_s;             /* dim values per entry, seen from the cell */
    const double* q0;        /* [nq][n_cells] initial state (may be NULL) */
    double gamma, Rgas, rhoInf, EInf, pInf, TInf, UInf[3], mu, Cp, PrInv;
    const double* rkA;       /* [rk_order] */
    const double* rkB;
    /* Processor-face halos of one partition of a decomposed case (0 for a
     * whole case): halo h is the neighbour slot N = n_cells + n_ghosts + h of
     * a processor face; each stage it takes the state of cell
     * halo_src_cell[h] of partition halo_src_part[h] (the reference receives
     * it over MPI, src/cfd_v0.cpp:3283-3374). */
    int64_t n_halos;
    const int64_t* halo_src_part;  /* [n_halos] */
    const int64_t* halo_src_cell;  /* [n_halos] solver-order cell of that partition */
    /* Boundary patch (index in the mesh's patch list) of each ghost, for the
     * wall-force post-processing (may be NULL: lfm_solver_forces is then
     * unavailable). */
    const int32_t* ghost_patch;    /* [n_ghosts] */
    /* Smagorinsky LES (turbulenceProperties simulationType other than
     * laminar; calc_VIS_Smagorinsky, src/cfd_v0.cpp:1573-1737): each cell's
     * model constant -2 (0.16 (1/vol_inv)^(1/3))^2, or NULL for laminar. */
    const double* smag_c;          /* [n_cells] */
} lfm_solver_desc;

typedef struct lfm_case lfm_case;
typedef struct lfm_solver lfm_solver;

/* Last error message of the calling thread ("" when none). */
const char* lfm_last_error(void);
/* Library version string. */
const char* lfm_version(void);

/* ---- case input (replaces CInputReader::initialize, src/inputReader.cpp:7-69,
 * and the polyMeshReaderOF / dictReaderOF / runTimeManagerOF plugins) ------ */

/* Reads an OpenFOAM case: <root>/system/{controlDict,fvSchemes},
 * <root>/constant/{spongeDict,thermophysicalProperties,turbulenceProperties},
 * the polyMesh of <root> (rank < 0) or <root>/processor<rank>, and the fields
 * p, T, U, alpha at the start time. */
int lfm_case_open(const char* root, int rank, lfm_case** out);

/* In-memory polyMesh and parameters (same meaning as the case files). */
typedef struct lfm_polymesh {
    int64_t n_points;
    const double* points;            /* [n_points][3] interleaved */
    int64_t n_faces;
    const int64_t* face_offsets;     /* [n_faces+1] */
    const int64_t* face_points;
    const int64_t* owner;            /* [n_faces] */
    int64_t n_internal_faces;
    const int64_t* neighbour;        /* [n_internal_faces] */
    int n_patches;
    const char* const* patch_name;
    const char* const* patch_type;   /* wall, patch, empty, cyclic, farfield ... */
    const int64_t* patch_start;
    const int64_t* patch_size;
    const char* const* patch_neighbour; /* cyclic partner name or NULL */
    const int64_t* cell_submesh;     /* optional [n_cells] or NULL */
    int64_t n_cells;
} lfm_polymesh;

typedef struct lfm_params {
    int solver, dimension, rk_order, minmod, laminar, residuals;
    double p_inf, T_inf, U_inf[3], Ls, mach, k_sponge;
    double Cp, mol_weight, mu, Pr;
    /* Solver order of the cells inside each submesh, for locality of the
     * device gathers: LFM_RENUMBER_NONE (polyMesh order, the reference's),
     * _RCM (reverse Cuthill-McKee), _HILBERT (Hilbert curve through the
     * cell centres) or _HPATH (the reference's Hamiltonian path).
     * lfm_case_open reads it from controlDict lfm/renumber
     * (none | rcm | hilbert | hpath). Written fields keep the polyMesh
     * numbering. */
    int renumber;
} lfm_params;

#define LFM_RENUMBER_NONE 0
#define LFM_RENUMBER_RCM 1
#define LFM_RENUMBER_HILBERT 2
/* The reference's Hamiltonian-path order (its hpath renumberMesh method,
 * hpathRenumber/hpathRenumber.C:127-180; designed for 2D meshes): boundary
 * cells as one walk, then the interior cells as another. */
#define LFM_RENUMBER_HPATH 3

typedef struct lfm_fields {
    const double* p;      /* [n_cells] */
    const double* T;      /* [n_cells] */
    const double* U;      /* [n_cells][3] interleaved */
    const double* alpha;  /* [n_cells] sponge distance, may be NULL when Ls <= 0 */
} lfm_fields;

int lfm_case_from_polymesh(const lfm_polymesh* mesh, const lfm_params* params, const lfm_fields* fields,
                           lfm_case** out);
/* Pointers into the case's arrays; valid until lfm_case_free. */
int lfm_case_describe(const lfm_case* c, lfm_solver_desc* out);
/* Run control read from controlDict: deltaT, endTime, writeInterval ... */
int lfm_case_time(const lfm_case* c, double* delta_t, double* start_time, double* end_time, int* adjust_time_step,
                  double* max_co);
/* polyMesh label of each solver-order cell ([n_cells]). */
int lfm_case_cell_ids(const lfm_case* c, int64_t* out);
void lfm_case_free(lfm_case* c);

/* ---- device solver (replaces ISolver, api/cfdv0_solver.h:18-105) -------- */

typedef struct lfm_solver_opts {
    int precision;        /* LFM_FP64 or LFM_FP32_BULK */
    int device;           /* CUDA device ordinal */
    int block;            /* threads per block for the cell/face kernels, 0 = default */
} lfm_solver_opts;

/* Uploads the description; the state starts at desc->q0 (or zero). */
int lfm_solver_create(const lfm_solver_desc* desc, const lfm_solver_opts* opts, lfm_solver** out);
void lfm_solver_destroy(lfm_solver* s);

/* Host <-> device state copies ([nq][n_cells], pageable or pinned host memory).
 * set_state also clears the non-finite flag that lfm_solver_sync reports. */
int lfm_solver_set_state(lfm_solver* s, const double* q);
int lfm_solver_get_state(lfm_solver* s, double* q);

/* One RK stage: prepare_for_RKstep, set_boundary_conditions, calc_gradients
 * (M2AUSM only), calc_VIS, one_rk_step_M* (src/mesh_solver.cpp:500-672).
 * Stage 0 also performs prepare_for_timestep. Asynchronous on the solver stream. */
int lfm_solver_stage(lfm_solver* s, int rk_stage, double dt);

/* nsteps full time steps at constant dt (rk_order stages each), replayed from
 * a CUDA graph. Asynchronous on the solver stream. */
int lfm_solver_step(lfm_solver* s, int nsteps, double dt);
/* Host state in, nsteps time steps, host state out, in one call with one
 * synchronisation at the end: q_in (may be NULL: continue from the device
 * state) is uploaded as by lfm_solver_set_state, q_out (may be NULL) receives
 * the state as from lfm_solver_get_state ([nq][n_cells], solver order, host
 * memory; pinned memory copies fastest). Returns lfm_solver_sync's status. */
int lfm_solver_advance(lfm_solver* s, const double* q_in, int nsteps, double dt, double* q_out);

/* Same as lfm_solver_step, timed with CUDA events on the solver stream;
 * waits for completion and returns the elapsed milliseconds. */
int lfm_solver_step_timed(lfm_solver* s, int nsteps, double dt, float* ms);

/* compute_cfl / compute_dt (src/cfd_v0.cpp:2886-2942) reduced on the device
 * deterministically; blocks until the value is on the host. */
int lfm_solver_cfl(lfm_solver* s, double dt, double* cfl);
int lfm_solver_min_dt(lfm_solver* s, double max_co, double* dt);

/* Sum over cells of the squared stage-0 residual of the last time step,
 * per conserved variable ([nq]); requires desc->residuals. */
int lfm_solver_residual(lfm_solver* s, double* res);

/* Per-cell stage-0 residual of the last time step, sum over the cell's faces
 * of the face rhs ([nq][n_cells], solver order): the RES of
 * updateSolutionResidual (src/cfd_v0.cpp:2973-2993). Requires desc->residuals. */
int lfm_solver_cell_residual(lfm_solver* s, double* res);

/* Cell residuals of a caller-supplied state without allocating anything.
 * This entry point has no counterpart in the reference. It is for callers
 * that must not allocate device memory at the time of the call: code running
 * while a CUDA graph is being captured, allocator-free real-time or serving
 * loops, and hosts whose device memory is owned by another runtime.
 *
 * q:   device pointer, [nq][q_stride] doubles (cells 0..n_cells-1 in solver
 *      order); read only.
 * res: device pointer, [nq][n_cells] doubles; receives, per cell, the sum over
 *      its faces of the face rhs for state q - the quantity that
 *      lfm_solver_cell_residual reports for the state at the start of a step.
 * stream: cudaStream_t to run on (NULL: the legacy default stream).
 * The solver handle supplies the geometry already on the device; its own
 * buffers and stream are not touched. Scratch (ghost states, primitives,
 * viscous terms, face rhs) lives in one static device array of
 * LFM_NOALLOC_SCRATCH_BYTES per GPU, held from the library's load until the
 * process exits; cases that need more return LFM_ERR_UNSUPPORTED, and so
 * does a partition of a decomposed case (a solver from
 * lfm_partitioned_solver): its processor-face halo states come from the
 * other partitions, which a caller's state q does not cover. The first
 * call on a device looks up that array's device address (set-up), so make it
 * before any stream capture. All calls share the array: calls whose work
 * overlaps on the GPU race with each other. */
#define LFM_NOALLOC_SCRATCH_BYTES (32u << 20)
int lfm_solver_residual_noalloc(const lfm_solver* s, const double* q, int64_t q_stride, double* res, void* stream);

/* ---- post-processing on the device ------------------------------------- */

/* Pressure statistics (haveAverage; postProcAverage and updateAverageField,
 * src/cfd_v0.cpp:3083-3104, 2966-2970). reset zeroes the per-cell sums;
 * accumulate(n) adds, from the current state, pAVG += p and
 * pRMS += (p - pAVG / n)^2 in every cell (nothing when n < 1: the reference
 * passes the step count since tStartAverage); get(n) returns
 * p_avg = pAVG * (1/n) and p_rms = sqrt(pRMS * (1/n)) per cell ([n_cells],
 * solver order). Asynchronous on the solver stream, except get. */
int lfm_solver_stats_reset(lfm_solver* s);
int lfm_solver_stats_accumulate(lfm_solver* s, int n);
int lfm_solver_stats_get(lfm_solver* s, int n, double* p_avg, double* p_rms);

/* Pressure and viscous forces on boundary patches (haveForces;
 * postProcForces, src/cfd_v0.cpp:3169-3250): for patch patches[i] (index in
 * the mesh's patch list, see desc->ghost_patch),
 *   f_pressure[i*dim + k] = sum over its faces of S_k (p - p_inf),
 *   f_viscous[i*dim + k]  = - sum over its faces of (tau . S)_k,
 * tau from the wall-normal velocity difference between the cell and its
 * ghost, summed in the reference's face order. The ghost state is, as the
 * reference's ghost cells hold after a step, the boundary state of the last
 * stage's starting state (the FP32-bulk path recovers that state from the
 * last update, q' - B dq); before any stage, that of the current state.
 * Synchronous. */
int lfm_solver_forces(lfm_solver* s, int n_patches, const int32_t* patches, double* f_pressure, double* f_viscous);

/* Pressure probes: p - p_inf of the listed cells (solver order), appended to
 * a device history by each record call (up to `capacity` records), read
 * back in one copy ([n_records][n]). */
int lfm_solver_probes_set(lfm_solver* s, int n, const int64_t* cells, int capacity);
int lfm_solver_probes_record(lfm_solver* s);
int lfm_solver_probes_read(lfm_solver* s, double* out, int* n_records);

/* Blocks until all work on the solver stream has finished and reports the
 * first CUDA or numeric error. */
int lfm_solver_sync(lfm_solver* s);

/* Writes `bytes` of device scratch memory on the solver stream so that the
 * next step starts with a cold L2 cache (benchmark timing aid). */
int lfm_solver_flush_l2(lfm_solver* s, size_t bytes);

/* Benchmark loop: nsteps time steps, each preceded by a write of flush_bytes
 * of scratch memory (outside its timing) and bracketed by events on the
 * solver stream; one synchronisation at the end. ms[k] = duration of step k. */
int lfm_solver_bench(lfm_solver* s, int nsteps, double dt, size_t flush_bytes, float* ms);

/* Device kernels launched per time step (for launch accounting). */
int lfm_solver_launches_per_step(const lfm_solver* s, int* launches);

/* Per-kernel times of one time step ([n] entries, ms summed over the RK
 * stages, names in lfm_solver_kernel_name), by prefix differences: the graph
 * of the step's first m kernel launches is timed (median of a few launches,
 * each after an L2 eviction when lfm_solver_bench has allocated its scrub
 * buffer) for every m, and the m-th launch is charged the difference. Each
 * kernel is so timed where it runs in the step, and the times add up to the
 * step's. Advances the state by partial steps. Synchronizes. */
int lfm_solver_profile_step(lfm_solver* s, double dt, int n, float* ms);
const char* lfm_solver_kernel_name(int i);

/* Flux kernel of an FP32-bulk solver (no reference counterpart: the
 * reference evaluates its faces in one loop). Every variant gives the same
 * bits; they differ in how a face's values reach the SM:
 *   LFM_FLUX_FACE    one thread per face;
 *   LFM_FLUX_CELL    one thread per cell over the faces it owns, the cell's
 *                    own rows read once (the default for 3D cases);
 *   LFM_FLUX_STAGED  the values each face reads copied into shared memory
 *                    ahead of use with cp.async: staging_depth buffers per
 *                    thread (1: one slot beside the registers; 2..4: chunks
 *                    of staging_faces faces per block, 32..256).
 * The variants apply to M1 / M2 laminar solvers with separate flux and update
 * kernels; other solvers report LFM_FLUX_FACE and refuse the others. */
#define LFM_FLUX_FACE 0
#define LFM_FLUX_CELL 1
#define LFM_FLUX_STAGED 2
typedef struct lfm_solver_tuning {
    int flux_kernel;     /* LFM_FLUX_* */
    int staging_depth;   /* LFM_FLUX_STAGED: shared-memory buffers per thread, 1..4 */
    int staging_faces;   /* LFM_FLUX_STAGED: faces per block, 32..256 (depth 1: 256) */
    float ms_per_step;   /* lfm_solver_autotune: median time step of the trial */
} lfm_solver_tuning;
int lfm_solver_get_tuning(const lfm_solver* s, lfm_solver_tuning* t);
/* Waits for the solver stream; LFM_ERR_UNSUPPORTED where the variant does not
 * apply, LFM_ERR_INVALID for a staged shape the device refuses (shared memory). */
int lfm_solver_set_tuning(lfm_solver* s, const lfm_solver_tuning* t);
/* Times trial_steps steps (after one untimed step, each after a write of
 * flush_bytes of scratch memory) of every applicable flux kernel
 * configuration -- the face and cell kernels and the staged kernel at depths
 * 1..4 -- and keeps the fastest (*chosen, with its median time); the state is
 * restored afterwards. tried[0..capacity) receives every configuration timed,
 * *n_tried their count (either may be NULL; configurations the device refuses
 * are skipped). Synchronous; copies the stored state on the device (device
 * memory for one copy of it) and puts it back bit for bit. */
int lfm_solver_autotune(lfm_solver* s, double dt, int trial_steps, size_t flush_bytes, lfm_solver_tuning* chosen,
                        lfm_solver_tuning* tried, int capacity, int* n_tried);

/* ---- decomposed cases on one GPU ------------------------------------------
 *
 * The reference runs a decomposed case (processor0..N-1, decomposePar) as one
 * MPI rank per partition, exchanging halo cells over MPI (MPI_env,
 * src/mpi_env.cpp:406-463; CFDv0_solver::mpi_communication/mpi_wait,
 * src/cfd_v0.cpp:3546-3603). Here all partitions run on one GPU: each
 * processor face's neighbour is a halo slot, and the exchange is an on-device
 * copy from the source partition -- conserved state before each stage,
 * viscous terms before the fluxes -- with no collective. */
typedef struct lfm_pcase lfm_pcase;
typedef struct lfm_partitioned lfm_partitioned;

/* Reads <root>/processor0..nparts-1 (polyMesh with processor patches and
 * faceProcAddressing / cellProcAddressing, fields at the start time) and the
 * dictionaries of <root>; builds every partition's description with its
 * halos resolved. */
int lfm_pcase_open(const char* root, int nparts, lfm_pcase** out);
int lfm_pcase_parts(const lfm_pcase* pc, int* nparts);
/* Partition part's description (pointers valid until lfm_pcase_free). */
int lfm_pcase_describe(const lfm_pcase* pc, int part, lfm_solver_desc* out);
/* Global cell (cellProcAddressing) of each solver-order cell of a partition. */
int lfm_pcase_cell_global(const lfm_pcase* pc, int part, int64_t* out);
int lfm_pcase_time(const lfm_pcase* pc, double* delta_t, double* start_time, double* end_time,
                   int* adjust_time_step, double* max_co);
void lfm_pcase_free(lfm_pcase* pc);

/* One solver per partition on a shared stream; descs[p] carries partition
 * p's halos (halo_src_part, halo_src_cell). */
int lfm_partitioned_create(const lfm_solver_desc* const* descs, int nparts, const lfm_solver_opts* opts,
                           lfm_partitioned** out);
void lfm_partitioned_destroy(lfm_partitioned* P);
/* State of one partition ([nq][n_cells] of that partition, solver order). */
int lfm_partitioned_set_state(lfm_partitioned* P, int part, const double* q);
int lfm_partitioned_get_state(lfm_partitioned* P, int part, double* q);
/* nsteps time steps of every partition (one CUDA graph per step); asynchronous. */
int lfm_partitioned_step(lfm_partitioned* P, int nsteps, double dt);
int lfm_partitioned_sync(lfm_partitioned* P);
/* The solver of one partition (owned by P, valid until lfm_partitioned_destroy),
 * for its per-partition queries: lfm_solver_cfl / _min_dt / _residual /
 * _cell_residual / _stats_* / _forces / _probes_*. Advance partitions only
 * through lfm_partitioned_step: a partition stepped on its own would not
 * refresh its halos. */
int lfm_partitioned_solver(lfm_partitioned* P, int part, lfm_solver** out);

/* Diagnostic: the tiles of the fused FP32-bulk stage kernel for a
 * description (host only, no device): runs of up to tile_cells cells, halved
 * while their local cells exceed max_local; out = {tiles, largest local cell
 * count, largest local face count, local cells summed over the tiles, flux
 * faces summed over the tiles}. LFM_ERR_INVALID when the tiles cannot be
 * built (processor halos) or an index check fails. */
int lfm_tiles_stats(const lfm_solver_desc* d, int tile_cells, int max_local, int64_t* out);

/* Diagnostic: runs the FP32-bulk kernels' integer-pipe binary32 <-> binary64
 * conversions on the device over n bit patterns (host arrays) and returns
 * their results, for comparison with IEEE 754 conversions. */
int lfm_selftest_fp_convert(int64_t n, const uint32_t* f32_bits, const uint64_t* f64_bits, uint64_t* f64_of_f32,
                            uint32_t* f32_of_f64);

/* ---- batch engine: many cases, one persistent kernel per RK stage ---------
 *
 * No single reference call corresponds: the reference advances one case per
 * MPI job (Mesh::solve, src/mesh_solver.cpp:474-853). A batch advances any
 * number of independent cases -- uneven sizes, 2D and 3D, M1/M2/M2AUSM --
 * with the FP32-bulk arithmetic (LFM_FP32_BULK), each case at its own constant
 * dt. A time step of all cases is one CUDA graph: one persistent kernel per RK
 * stage whose blocks work through per-phase tile lists of every case, with
 * grid-wide barriers between the phases. Case data lives in one device arena
 * reserved at creation; a case is admitted when a free block of its footprint
 * exists (lfm_batch_case_bytes) and its block is returned on removal. Cases may
 * be added and removed between steps. Calls on one batch are not re-entrant;
 * all work runs on the batch's own stream. */
typedef struct lfm_batch lfm_batch;

typedef struct lfm_batch_opts {
    int device;           /* CUDA device ordinal */
    int rk_order;         /* RK stages per step, shared by every case (1..8) */
    size_t arena_bytes;   /* device memory reserved for case data; 0 = a quarter of free memory */
    int max_cases;        /* case slots; 0 = 256 */
} lfm_batch_opts;

/* Launch shape of the stage kernel, chosen by lfm_batch_autotune. */
typedef struct lfm_batch_tuning {
    int block;            /* threads per block: 128, 256 or 512 */
    int items_per_thread; /* cells or faces per thread and tile (tile = block x items) */
    int blocks_per_sm;    /* resident blocks per SM of the persistent grid; 0 = all that fit */
    int cooperative;      /* 1: cooperative launch (co-residency guaranteed by the driver) */
    /* 1: one kernel per phase instead of the persistent stage kernel (no
     * grid barriers; each phase at its own occupancy; blocks_per_sm then
     * caps each phase kernel's grid, 0 = all that fit) */
    int phased;
} lfm_batch_tuning;

int lfm_batch_create(const lfm_batch_opts* opts, lfm_batch** out);
void lfm_batch_destroy(lfm_batch* b);
/* Arena footprint of a case (bytes). */
int lfm_batch_case_bytes(const lfm_solver_desc* desc, size_t* bytes);
/* Admits a case with state desc->q0 and constant time step dt; *slot receives
 * its slot. LFM_ERR_NOMEM when no arena block or slot is free. */
int lfm_batch_add(lfm_batch* b, const lfm_solver_desc* desc, double dt, int* slot);
/* Removes a case (waits for queued steps) and frees its arena block. */
int lfm_batch_remove(lfm_batch* b, int slot);
/* Host <-> device state of one case ([nq][n_cells], solver order); synchronous.
 * set_state also clears the case's non-finite flag. */
int lfm_batch_set_state(lfm_batch* b, int slot, const double* q);
int lfm_batch_get_state(lfm_batch* b, int slot, double* q);
/* The cases slots[0..n) from host states q_in[i] ([nq][n_cells] as
 * lfm_batch_set_state; a NULL array or entry keeps that case's state), nsteps
 * steps of the batch, the states out into q_out[i] (NULL skips), all on the
 * batch stream with one synchronisation at the end; returns lfm_batch_sync's
 * status. Gives the bits of the separate calls. */
int lfm_batch_advance(lfm_batch* b, int n, const int* slots, const double* const* q_in, int nsteps,
                      double* const* q_out);
/* nsteps time steps of every case in the batch; asynchronous. */
int lfm_batch_step(lfm_batch* b, int nsteps);
/* Waits for the batch stream; LFM_ERR_NUMERIC names the slots whose state
 * became non-finite, LFM_ERR_CUDA reports a stage kernel that gave up at a
 * grid barrier. */
int lfm_batch_sync(lfm_batch* b);
/* LFM_OK or LFM_ERR_NUMERIC for one case (waits for the batch stream). */
int lfm_batch_case_status(lfm_batch* b, int slot, int* status);
/* Arena: largest free block, total free bytes, arena size (any may be NULL). */
int lfm_batch_memory(const lfm_batch* b, size_t* largest_free, size_t* total_free, size_t* arena_bytes);
/* Cells and cases currently in the batch (either may be NULL). */
int lfm_batch_cells(const lfm_batch* b, int64_t* cells, int* cases);
int lfm_batch_get_tuning(const lfm_batch* b, lfm_batch_tuning* t);
int lfm_batch_set_tuning(lfm_batch* b, const lfm_batch_tuning* t);
/* Times trial_steps steps of the current cases for every launch shape and
 * keeps the fastest; the cases' states are restored afterwards. */
int lfm_batch_autotune(lfm_batch* b, int trial_steps, lfm_batch_tuning* chosen);
/* nsteps steps, each after a write of flush_bytes of scratch (outside its
 * timing), ms[k] = duration of step k (CUDA events on the batch stream).
 * Reports barrier failures; numeric state is left to lfm_batch_sync and
 * lfm_batch_case_status. */
int lfm_batch_bench(lfm_batch* b, int nsteps, size_t flush_bytes, float* ms);
/* Kernel launches per time step (one per RK stage). */
int lfm_batch_launches_per_step(const lfm_batch* b, int* launches);
/* Failure-detection test aid, no reference counterpart: every grid barrier of
 * the persistent stage kernel then waits for extra_arrivals blocks more than
 * its grid has (0: normal operation). With extra_arrivals > 0 no barrier is
 * ever reached: each block gives up after its bounded wait (about a second),
 * the kernel returns, and lfm_batch_sync reports LFM_ERR_CUDA; the batch's
 * case states are then undefined. Affects the persistent launch mode only
 * (lfm_batch_tuning.phased = 0). */
int lfm_batch_debug_barrier(lfm_batch* b, int extra_arrivals);

/* ---- request server: continuous batching of solve requests ---------------
 *
 * No reference counterpart (the reference runs one case per job). A server
 * owns a batch and one worker thread. lfm_server_submit packs a request (a
 * case, its dt and step count) on the calling thread and queues it; the worker
 * admits queued requests in arrival order whenever a case slot and an arena
 * block of the request's footprint are free (a request that does not fit is
 * passed over at most max_bypass times before admission waits for it),
 * advances all admitted requests together in chunks of at most chunk_steps
 * steps, and retires finished requests (copying their state out and freeing
 * their slot and block) at chunk boundaries, where newly arrived requests
 * join. A request's result does not depend on what else runs beside it (the
 * batch computes every case with the same kernels). All functions are
 * thread-safe. Times are seconds on a steady clock since lfm_server_create. */
typedef struct lfm_server lfm_server;

typedef struct lfm_server_opts {
    int device;
    int rk_order;             /* RK stages per step of every request */
    size_t arena_bytes;       /* device memory for admitted requests; 0 = a quarter of free memory */
    int max_cases;            /* most requests on the device at once; 0 = 256 */
    int chunk_steps;          /* most steps between admission passes; 0 = 50 */
    int max_bypass;           /* times the oldest waiting request may be passed over; 0 = 8, < 0 = never */
    lfm_batch_tuning tuning;  /* launch shape of the stage kernel; block 0 = default */
    /* Requests of at least solo_cells cells (0: none) run on their own
     * FP32-bulk single-case solver instead of in the batch, at most max_solo
     * at once (0 = 2): the single-case kernels are faster than the batch's on
     * large cases, and a case gives the same bits either way. A second server
     * thread builds their solvers ahead of admission while the batch runs;
     * their device memory, outside the arena, is held from that build until
     * the request retires (at most max_solo built or running at once). */
    int64_t solo_cells;
    int max_solo;
} lfm_server_opts;

typedef struct lfm_request_info {
    int state;                /* 0 queued, 1 running, 2 done */
    int status;               /* LFM_OK, LFM_ERR_NUMERIC (non-finite state: the result is the state at
                                 detection), LFM_ERR_NOMEM (larger than the arena), other: server failure */
    int64_t cells;
    int steps;
    double t_submit, t_admit, t_done;   /* -1 when not reached */
    size_t footprint_bytes;
    int steps_done;           /* time steps advanced so far */
} lfm_request_info;

typedef struct lfm_server_stats {
    int queued, running;
    int64_t completed;
    int64_t chunks;           /* chunks of steps run so far */
    double t_now;
    double busy_s;            /* seconds the worker spent advancing chunks (launch to synchronisation) */
    double cell_stages;       /* cell-RK-stage updates advanced so far, finished requests or not */
} lfm_server_stats;

int lfm_server_create(const lfm_server_opts* opts, lfm_server** out);
/* Stops the worker (queued and running requests are abandoned) and frees the server. */
void lfm_server_destroy(lfm_server* s);
/* Queues nsteps steps of the case at time step dt, starting from desc->q0;
 * the description may be freed when the call returns. */
int lfm_server_submit(lfm_server* s, const lfm_solver_desc* desc, double dt, int nsteps, int64_t* id);
int lfm_server_info(lfm_server* s, int64_t id, lfm_request_info* info);
/* Waits until the request is done or timeout_s passes (< 0: no limit). */
int lfm_server_wait(lfm_server* s, int64_t id, double timeout_s, int* done);
/* Final state of a done request ([nq][n_cells], may be NULL) and its info;
 * releases the request. */
int lfm_server_result(lfm_server* s, int64_t id, double* q, lfm_request_info* info);
int lfm_server_get_stats(lfm_server* s, lfm_server_stats* st);

#ifdef __cplusplus
}
#endif
#endif
