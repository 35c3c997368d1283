/*
 * ebb_gb300.h -- C ABI of the GB300-native explicit unstructured finite-volume update.
 *
 * Every entry point is plain C: pointers, sizes and status codes, no C++ or torch
 * types.  The caller owns host buffers; the library owns device memory.  A solver
 * handle is bound to one CUDA stream and is not thread-safe; use one handle per
 * host thread.  Calls never abort the process and kernels never trap: failures
 * come back as an ebb_status, and ebb_last_error() gives the detail.
 *
 * Reference interfaces replaced (EbbCFD, D sources):
 *   ebb_config_parse       source/config.d:112-313   loadConfig(string) -> Config
 *   ebb_mesh_import        source/io.d:669-990       importMesh / parseGmshMesh (gmsh 2.2 ASCII)
 *   ebb_solver_create      source/mesh.d:217-643     UMesh2.buildMesh
 *                          source/solve.d:175-279    ufvmSetup (IC and BC binding)
 *   ebb_residual           source/solve.d:322-1122   ufvmSolver!(F,4)(R, q, mesh, config, newDt, Rmax, limit, dtUpdate)
 *   ebb_step               source/integrators.d:17-270  Euler/RK2/RK2_TVD/RK4.step!solver(R, q, mesh, config, dt, Rmax)
 *   ebb_run                app/solver.d:38-277       runIntegrator loop body (NaN check, RMS, forces, CFL adjust, dt/t)
 *   ebb_flux               source/flux.d:66-141,224-303  rusanovFlux!4 / roeFlux!4 (qL, qR, n, ref sMax)
 *   ebb_save_solution      source/io.d:68-161        saveSolution (.esln v2, big-endian)
 *   ebb_load_solution      source/io.d:218-366       loadSolution
 *   ebb_reconstruct        app/reconstruct.d:79-424  ebb-reconstruct (refined .mmsh / .esln)
 */
#ifndef EBB_GB300_H
#define EBB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EBB_ABI_VERSION 1
#define EBB_MAX_BC 32
#define EBB_MAX_FORCE_TAGS 8
#define EBB_TAG_LEN 64
#define EBB_PATH_LEN 1024
#define EBB_FLUX_NOALLOC_MAX 32768

typedef enum {
    EBB_OK = 0,
    EBB_ERR_ARG = 1,        /* bad argument or handle */
    EBB_ERR_IO = 2,         /* file could not be opened/read/written */
    EBB_ERR_FORMAT = 3,     /* malformed gmsh / JSON / .esln */
    EBB_ERR_MESH = 4,       /* mesh topology/geometry rejected (e.g. non-positive area) */
    EBB_ERR_CONFIG = 5,     /* config inconsistent with mesh (e.g. missing BC tag) */
    EBB_ERR_CUDA = 6,       /* CUDA runtime failure */
    EBB_ERR_OOM = 7,        /* device allocation failed */
    EBB_ERR_NAN_EDGE = 8,   /* NaN face flux (reference: EdgeException, solve.d:806-1076) */
    EBB_ERR_NAN_CELL = 9,   /* NaN cell state after a step (reference: CellException, app/solver.d:131-149) */
    EBB_ERR_NO_DEVICE = 10, /* no CUDA device / extension not usable */
    EBB_ERR_BC = 11,        /* boundary condition failed (tpInflow: both Mach roots negative, solve.d:662-669) */
    EBB_ERR_LIMIT = 12      /* size beyond a documented limit */
} ebb_status;

/* boundary types, same order as enum BoundaryType (source/mesh.d:27-36) */
typedef enum {
    EBB_BC_FULL_STATE = 0,
    EBB_BC_CONST_PRESSURE = 1,
    EBB_BC_INVISCID_WALL = 2,
    EBB_BC_VISCOUS_WALL = 3,
    EBB_BC_SYMMETRY = 4,
    EBB_BC_TEMP_PRES_INFLOW = 5,
    EBB_BC_DIRICHLET = 6
} ebb_bc_type;

/* flux names of fluxList (source/flux.d:12) */
typedef enum { EBB_FLUX_RUSANOV = 0, EBB_FLUX_ROE = 1 } ebb_flux_kind;
/* integrator names of integratorList (source/integrators.d:17) */
typedef enum { EBB_INT_EULER = 0, EBB_INT_RK2 = 1, EBB_INT_RK2_TVD = 2, EBB_INT_RK4 = 3 } ebb_integrator;

/* precision forms */
typedef enum {
    EBB_PREC_FP64 = 0,  /* plain FP64 path, same operation order as the reference */
    EBB_PREC_SPLIT = 1, /* FP32 flux/gradient/limiter arithmetic, FP64 geometry, state update and reductions */
    EBB_PREC_DF = 2     /* flux/gradient/limiter arithmetic on double-floats (pairs of FP32 numbers, ~46
                           significant bits) on the FP32 pipe; FP64 geometry, state update and reductions */
} ebb_precision;

/* manufactured-solution fields used by Dirichlet boundaries and the source term */
typedef enum {
    EBB_MMS_NONE = 0,
    EBB_MMS_REFERENCE = 1, /* source/manufacturedsolution.d:27-282 */
    EBB_MMS_SINE = 2       /* rho=1+0.1 sin(2pi x)cos(2pi y), u=0.5+0.05 cos(2pi x)sin(2pi y),
                              v=0.3+0.05 sin(2pi x+1), p=1/1.4+0.1 cos(2pi y) (Euler source) */
} ebb_mms;

typedef struct {
    char tag[EBB_TAG_LEN];
    int32_t type;   /* ebb_bc_type */
    int32_t n_data; /* entries of "q" */
    double data[8];
} ebb_boundary;

/* struct Config (source/config.d:72-94), flattened. */
typedef struct {
    char mesh_file[EBB_PATH_LEN];
    double dt;
    int32_t dynamic_dt;
    double t_end;
    int32_t flux; /* ebb_flux_kind */
    int64_t save_iter;
    int64_t plot_iter;
    int32_t n_force;
    char force_boundary[EBB_MAX_FORCE_TAGS][EBB_TAG_LEN];
    int32_t integrator; /* ebb_integrator */
    int32_t limited;
    double lp_thresh;
    int64_t order;
    double cfl;
    double ic[4]; /* M, aoa (deg), p (unused), rho */
    int32_t n_boundaries;
    ebb_boundary boundaries[EBB_MAX_BC];
    int32_t local_timestep;
    int32_t multistage_limiting;
    int32_t cfl_adjust;
    int32_t viscosity;
    double pr, r_gas, gamma, mu, re, l_ref; /* physicalConfig; gamma is parsed but 1.4 is used (euler.d:89) */
    int32_t mms;                            /* ebb_mms; 0 for ebb-solve configs */
} ebb_config;

typedef struct ebb_mesh ebb_mesh;
typedef struct ebb_solver ebb_solver;

typedef struct {
    int64_t n_nodes;
    int64_t n_cells;      /* interior cells (elements) */
    int64_t n_ghost;      /* boundary edges = ghost cells */
    int64_t n_edges;      /* interior + boundary edges */
    int64_t n_int_edges;
    int32_t n_tags;
    int32_t max_edges;    /* largest element edge count */
    int64_t face_slots;   /* sum of element edge counts */
} ebb_mesh_info;

/* per-step record of ebb_run (the quantities app/solver.d:178-230 prints and writes) */
typedef struct {
    double t;      /* time before the increment (the .frc time column) */
    double drag;   /* ld[0] */
    double lift;   /* ld[1] */
    double resid[4];
    double rmax;   /* Flux_R */
    double dt;     /* dt after the step's update */
    double cfl;
} ebb_step_record;

/* ---- library ---------------------------------------------------------- */
int ebb_abi_version(void);
/* sizeof the public structs, for FFI bindings to check their layout */
int ebb_struct_sizes(size_t *config, size_t *mesh_info, size_t *step_record);
/* Returns EBB_OK when a CUDA device is usable (sets *n_devices). */
int ebb_device_count(int *n_devices);
/* Select the device later solver handles are created on (one GPU per process). */
int ebb_set_device(int device);
/* Page-locked host buffers for fast state copies (cudaMallocHost / cudaFreeHost).  A
   state upload (ebb_set_state, ebb_batch_set_state) whose array starts on a 16-byte
   boundary inside such a buffer is read by the device directly, with no staging copy;
   any other host array is staged through device memory.  The buffer must stay
   allocated for the duration of the call only. */
int ebb_host_alloc(size_t bytes, void **ptr);
int ebb_host_free(void *ptr);

/* ---- config (source/config.d:112-313) ---------------------------------- */
void ebb_config_defaults(ebb_config *cfg);
int ebb_config_parse(const char *json_text, ebb_config *out, char *err, size_t err_len);

/* ---- mesh (source/io.d:669-990) ---------------------------------------- */
int ebb_mesh_import(const char *path, ebb_mesh **out, char *err, size_t err_len);
/* Build from arrays: xy[2*n_nodes]; elem_off[n_elem+1]; elem_nodes 1-based node
   numbers (any orientation; clockwise elements are reversed as io.d:969-987 does);
   b_nodes[2*n_b] 0-based; b_group_start[n_tags]; tags as n_tags NUL-terminated strings
   packed at stride EBB_TAG_LEN. */
int ebb_mesh_from_arrays(int64_t n_nodes, const double *xy, int64_t n_elem, const int64_t *elem_off,
                         const int32_t *elem_nodes, int64_t n_b, const int32_t *b_nodes, int32_t n_tags,
                         const int64_t *b_group_start, const char *tags, ebb_mesh **out, char *err, size_t err_len);
int ebb_mesh_get_info(const ebb_mesh *mesh, ebb_mesh_info *info);
int ebb_mesh_get_tag(const ebb_mesh *mesh, int32_t i, char *tag, size_t len);
/* element centroids in reference cell order (cx, cy), for initial conditions and error norms */
int ebb_mesh_centroids(const ebb_mesh *mesh, double *xy);
/* The reference's edges (mesh.d:242-313: creation order, interior and boundary mixed),
   n_edges of them: group[e] = boundary tag index or -1 for an interior edge;
   cells[2e], cells[2e+1] = cellIdx[0] (the creating element) and cellIdx[1] (the other
   element, or n_cells + ghost index on a boundary); mid, normal (2 per edge, pointing
   out of cellIdx[0]) and len.  Any output may be NULL. */
int ebb_mesh_edges(const ebb_mesh *mesh, int32_t *group, int32_t *cells, double *mid, double *normal, double *len);
void ebb_mesh_free(ebb_mesh *mesh);

/* ---- solver (buildMesh + ufvmSetup) ------------------------------------ */
int ebb_solver_create(const ebb_mesh *mesh, const ebb_config *cfg, int32_t precision, ebb_solver **out, char *err,
                      size_t err_len);
void ebb_solver_destroy(ebb_solver *s);
int ebb_last_error(const ebb_solver *s, int32_t *kind, int64_t *index, char *msg, size_t msg_len);

/* state in reference cell order, q[n_cells][4] */
int ebb_set_state(ebb_solver *s, const double *q);
int ebb_get_state(ebb_solver *s, double *q);
int ebb_get_time(ebb_solver *s, double *t, double *dt, int64_t *iterations);
int ebb_set_time(ebb_solver *s, double t, double dt);

/* One residual evaluation (ufvmSolver, plus the manufactured source when cfg.mms != 0)
   on host state q[n_cells][4]; writes R[n_cells][4]; *new_dt is the CFL time step and
   *rmax = max(*rmax, max|sum of len*flux|) as solve.d:1080-1121. */
int ebb_residual(ebb_solver *s, const double *q, double *R, double *new_dt, double *rmax, int32_t limit,
                 int32_t dt_update);
/* Same on device buffers already laid out by the solver (q_dev/R_dev hold n_cells x 4
   doubles in reference order); no host copies. */
int ebb_residual_device(ebb_solver *s, const double *q_dev, double *R_dev, double *new_dt, double *rmax,
                        int32_t limit, int32_t dt_update);

/* One integrator step on the resident state with time step *dt; on return *dt is the
   next step's CFL time step and *rmax the step's Flux_R (integrators.d). */
int ebb_step(ebb_solver *s, double *dt, double *rmax);

/* Up to max_steps iterations of the runIntegrator loop (stops at t >= tEnd).  Records
   (may be NULL) receive one entry per step run; *steps_run the count. */
int ebb_run(ebb_solver *s, int64_t max_steps, ebb_step_record *records, int64_t *steps_run);

/* ebb_run without records, also returning the device time of the launched steps
   measured with CUDA events on the solver's stream (no host synchronisation between
   the events). */
int ebb_run_timed(ebb_solver *s, int64_t max_steps, int64_t *steps_run, double *device_ms);

/* Face states of the last residual evaluation per cell and local edge, reference order
   (the edge values .esln v2 stores, io.d:111-133): out[face_slots][4]. */
int ebb_get_face_states(ebb_solver *s, double *out);

/* len * flux of every edge from the last residual evaluation, at its reference edge id
   (ebb_mesh_edges order): out[n_edges][4].  These are the terms the residual sums and
   computeBoundaryForces adds up over the force tags (mesh.d:645-671: edge.flux * len),
   e.g. the wall shear of a viscous wall is out[e][1] / len.  Single solves only
   (EBB_ERR_ARG for a batched arena). */
int ebb_get_edge_fluxes(ebb_solver *s, double *out);

/* The CUDA stream (cudaStream_t) the solver launches on, for callers that time or
   order work around it with CUDA events. */
int ebb_get_stream(ebb_solver *s, void **stream);
/* Average device time (ms, CUDA events on the solver stream) of each kernel of one
   first-stage pass on the resident state, over n_rep launches each:
   ms[0] cell (gradients, limiters, face states), ms[1] flux, ms[2] residual/update,
   ms[3] step end.  The state is left as it was. */
int ebb_profile_kernels(ebb_solver *s, int32_t n_rep, double *ms);

/* ---- batched arena (no counterpart in the reference: its driver runs one mesh per
   process) ----------------------------------------------------------------- */
/* n independent solves, each a mesh + config as for ebb_solver_create, laid out in one
   device arena and advanced together: each kernel of a stage is one launch over the
   cells and faces of every instance.  The instances must agree on flux, integrator,
   limiter, order, viscosity and MMS kind (EBB_ERR_CONFIG otherwise); meshes, boundary
   data, Mach, Reynolds, CFL, dt and tEnd may differ.  The handle takes the ebb_solver
   calls: ebb_set_state / ebb_get_state move the instances' states concatenated in
   instance order (ebb_batch_status gives each instance's offset); ebb_run advances
   every instance that is not done until all are done or max_steps have run, and
   writes no records when n > 1.  Each instance stops by itself at its tEnd, its step
   limit or its residual drop (ebb_batch_set_stop), or at its first NaN, which halts
   that instance only.  ebb_get_time / ebb_set_time / ebb_load_solution act on
   instance 0; ebb_residual, ebb_residual_device and ebb_step return EBB_ERR_ARG when
   n > 1.  Every instance's results are bitwise those of its own single solve. */
int ebb_batch_create(int32_t n, const ebb_mesh *const *meshes, const ebb_config *cfgs, int32_t precision,
                     ebb_solver **out, char *err, size_t err_len);

typedef struct ebb_instance_status {
    int64_t cell_offset; /* first row of the instance in ebb_get_state / ebb_set_state arrays */
    int64_t n_cells;
    int64_t iterations;
    double t, dt, cfl;
    int32_t done;      /* stopped: tEnd, step limit, residual drop, or an error */
    int32_t status;    /* EBB_OK, or the error that stopped it */
    int64_t err_index; /* reference index (within the instance) of the failing edge or cell, or -1 */
    double drag, lift, resid[4], rmax; /* of the latest iteration */
    double resid_first;                /* density residual of the first iteration (-1 before it) */
} ebb_instance_status;

int ebb_batch_size(const ebb_solver *s, int32_t *n);
/* status of instances first .. first+count-1 (one device-to-host copy) */
int ebb_batch_status(ebb_solver *s, int32_t first, int32_t count, ebb_instance_status *out);
/* Stop conditions of instance k (every instance for k < 0): tEnd; a step limit
   (max_steps > 0: done after that many iterations); a residual drop (resid_drop > 0:
   done once the density residual resid[0] <= resid_drop x its first-iteration value;
   the density residual is the one of the four whose normalising sum cannot vanish). */
int ebb_batch_set_stop(ebb_solver *s, int32_t k, double t_end, int64_t max_steps, double resid_drop);
/* state of instance k alone, q[n_cells_k][4] in that mesh's reference cell order */
int ebb_batch_get_state(ebb_solver *s, int32_t k, double *q);
int ebb_batch_set_state(ebb_solver *s, int32_t k, const double *q);
/* Enqueue n_steps iterations on the handle's stream and return without waiting
   (instances already done skip their work); ebb_batch_status or ebb_sync waits. */
int ebb_launch_steps(ebb_solver *s, int64_t n_steps);
int ebb_sync(ebb_solver *s);
/* device bytes ebb_batch_create would allocate for these meshes, without a device */
int ebb_batch_footprint(int32_t n, const ebb_mesh *const *meshes, const ebb_config *cfgs, int32_t precision,
                        size_t *bytes, char *err, size_t err_len);

/* ---- request server (no counterpart in the reference) ---------------------
   A continuous-batching loop over batched arenas.  Submitted solves are laid out on
   host threads; each scheduling round (ebb_server_tick) retires instances that have
   stopped (tEnd, step limit, residual drop or an error) and keeps their final states
   until fetched, frees arenas whose instances have all stopped, admits waiting
   requests into new arenas while their device bytes fit the budget (oldest first,
   grouped with waiting requests of the same physics and similar size), and advances
   every arena on its own stream so that arenas overlap on the device.  A request's
   results are bitwise those of solving it alone with the same stop conditions. */
typedef struct ebb_server ebb_server;

typedef struct ebb_server_options {
    int32_t precision;     /* EBB_PREC_FP64, EBB_PREC_SPLIT or EBB_PREC_DF (default split) */
    int32_t max_arenas;    /* arenas on the device at once (default 32) */
    int32_t max_batch;     /* instances per arena at most (default 512) */
    int32_t build_threads; /* host threads laying out submitted meshes (default 4) */
    double tick_ms;        /* device time each arena is given per round (default 25 ms) */
    double size_ratio;     /* cell counts grouped in one arena differ by at most this factor (default 4) */
    int64_t arena_cells;   /* cells per arena at most (default 8M) */
    uint64_t hbm_budget;   /* device bytes all arenas together may take (default 150e9) */
    int32_t escalate;      /* 1: a split-precision solve that stops with an error is solved
                              again in plain FP64 from its initial state (default 0) */
    int32_t finish_fp64;   /* 1: a split-precision solve with a residual drop whose density
                              residual, after falling at least 1000-fold from its first
                              iteration, makes no new minimum for stall_steps iterations (it
                              has levelled off at the FP32 rounding of its increments) continues in
                              finish_precision from its current state -- same id, iteration
                              count, time and first-iteration residual -- until the drop, its
                              step limit or tEnd (default 1) */
    int32_t stall_steps;   /* default 1000 */
    int32_t finish_precision; /* form of that continuation: EBB_PREC_FP64 (default) or
                                 EBB_PREC_DF (double-float: about 4.7x FP64's speed on the
                                 4.0M-cell viscous plate, within ~1e-10 of its forces) */
} ebb_server_options;

typedef struct ebb_request_result {
    int64_t id;
    int32_t status; /* EBB_OK, or the error that ended the solve */
    int32_t done_reason; /* 0 error, 1 tEnd, 2 step limit, 3 residual drop */
    int64_t err_index;
    int64_t n_cells;
    int64_t iterations;
    double t, drag, lift, resid[4], resid_first;
    double submit_s, admit_s, finish_s; /* server clock: seconds since ebb_server_create */
    int32_t precision;                  /* precision form of the solve that produced the result */
    int32_t escalated;                  /* 1: re-solved in FP64 after a split-precision error;
                                           2: finished in the finishing form (precision) after
                                              its split solve stalled */
    int64_t split_iterations;           /* iterations run in split precision */
    char msg[96];
} ebb_request_result;

typedef struct ebb_server_stats {
    uint64_t bytes_in_use, bytes_peak;
    int32_t arenas, waiting, building, reserved;
    int64_t submitted, finished, cell_updates, escalations;
} ebb_server_stats;

void ebb_server_options_defaults(ebb_server_options *o);
int ebb_server_create(const ebb_server_options *o, ebb_server **out, char *err, size_t err_len);
/* Queue one solve: mesh and config are copied (the caller may free them on return);
   it stops after max_steps iterations (> 0), at a residual drop (> 0: density residual
   <= resid_drop x its first-iteration value) or at the config's tEnd, whichever first.
   Thread-safe against ebb_server_tick. */
int ebb_server_submit(ebb_server *sv, const ebb_mesh *mesh, const ebb_config *cfg, int64_t max_steps,
                      double resid_drop, int64_t *id);
/* One scheduling round; *n_active / *n_waiting (may be NULL) count arenas on the
   device and requests not yet admitted (including those still being laid out). */
int ebb_server_tick(ebb_server *sv, int32_t *n_active, int32_t *n_waiting);
/* Results of requests finished since the last call, up to cap; *n the count. */
int ebb_server_results(ebb_server *sv, ebb_request_result *out, int32_t cap, int32_t *n);
/* Final state of a finished request, q[n_cells][4] in its mesh's reference cell
   order; the server then releases it.  EBB_ERR_ARG for an unknown or taken id. */
int ebb_server_take_state(ebb_server *sv, int64_t id, double *q);
int ebb_server_stats_get(ebb_server *sv, ebb_server_stats *st);
void ebb_server_destroy(ebb_server *sv);

/* ---- flux seam (source/flux.d) ------------------------------------------ */
/* Batched device evaluation of rusanovFlux!4 / roeFlux!4 on host arrays:
   qL,qR[n][4], normal[n][2] -> F[n][4], s_max[n]. */
int ebb_flux(int32_t kind, int64_t n, const double *qL, const double *qR, const double *normal, double *F,
             double *s_max);
/* Same evaluation and results as ebb_flux, for callers that cannot allocate device
   memory when they call.  This variant has no counterpart in the reference.  ebb_flux
   allocates and frees device staging buffers on every call; a caller that shares the
   GPU with running solves cannot afford that (cudaFree synchronises the whole device
   and stalls every stream the solves run on), and in a process whose device memory is
   already reserved (a request server's HBM budget) the allocation fails.  This
   variant stages through one fixed array compiled into the library
   (EBB_FLUX_NOALLOC_MAX faces, 3.75 MiB held on every GPU that loads the library until
   the process exits) and returns EBB_ERR_LIMIT, touching no output, for n larger than
   EBB_FLUX_NOALLOC_MAX.  Its first call on a device sets up that device (the array's
   device address and a non-blocking stream the call runs on); make that first call
   before any stream capture.  Calls share the array, which keeps the last call's
   contents: calls that overlap on the same GPU race and must be serialised. */
int ebb_flux_noalloc(int32_t kind, int64_t n, const double *qL, const double *qR, const double *normal, double *F,
                     double *s_max);

/* ---- files ---------------------------------------------------------------- */
/* .esln v2 of the resident state with the header time t and step dt (saveSolution
   takes them as arguments: the time loop of app/solver.d saves before advancing t). */
int ebb_save_solution(ebb_solver *s, const char *path, double t, double dt);
int ebb_load_solution(ebb_solver *s, const char *path);
/* loadSolution of a partitioned run (io.d:218-366): every file's cells go to their
   global ids; t and dt come from the first file; EBB_ERR_FORMAT unless every cell is
   covered. */
int ebb_load_solution_parts(ebb_solver *s, int32_t n, const char *const *paths);

/* ---- ebb-reconstruct (app/reconstruct.d:79-424) ---------------------------
   One residual evaluation of the resident state (limited as the config's "limited",
   no time-step update) gives gradients, limiters and the states on both sides of
   every edge; the refined mesh then has, as points: the nodes the elements use (node
   order), the edge midpoints (reference edge order) and the cell centroids, each
   cell split into 2 x nEdges triangles; its values: node values (the average over
   the node's cells of the limited gradient extrapolation to the node; boundary nodes
   average the values of their boundary edges), edge values (mean of the edge's two
   states) and the cell averages.  mmsh_path / esln_path (may be NULL) receive the
   .mmsh and .esln files of the refined mesh (t, dt in the .esln header); q_out (may
   be NULL) receives the n_out x 4 values; with all three NULL only *n_out is set.
   The mesh is the one the solver was created from.  EBB_ERR_NAN_CELL (index = node)
   when a node value is NaN, as the reference refuses. */
int ebb_reconstruct(ebb_solver *s, const ebb_mesh *mesh, const char *mmsh_path, const char *esln_path, double t,
                    double dt, double *q_out, int64_t *n_out);

#ifdef __cplusplus
}
#endif
#endif
