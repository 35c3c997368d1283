/+
 + ebb.gb300 -- D binding of the GB300 solver library's C ABI (include/ebb_gb300.h).
 +
 + One declaration per header function and one struct per header struct, in the
 + header's field order, so that `extern(C)` calls from EbbCFD's D host (app/solver.d,
 + app/ms.d, app/reconstruct.d) reach libebbgb300.so directly.  Link with
 + `-L-L<dir of libebbgb300.so> -L-lebbgb300` (the library carries its CUDA runtime).
 + Check the struct layouts once at start-up with checkLayout().
 +
 + No D compiler is available where this binding was written, so it is shipped as
 + source and has not been compiled; a CPU test checks that it declares every
 + function of the header with the same parameter count and every struct with the
 + header's fields.
 +/
module ebb.gb300;

extern(C) @nogc nothrow:

enum EBB_ABI_VERSION = 1;
enum EBB_MAX_BC = 32;
enum EBB_MAX_FORCE_TAGS = 8;
enum EBB_TAG_LEN = 64;
enum EBB_PATH_LEN = 1024;
enum EBB_FLUX_NOALLOC_MAX = 32768;

// ebb_status
enum : int
{
    EBB_OK = 0,
    EBB_ERR_ARG = 1,
    EBB_ERR_IO = 2,
    EBB_ERR_FORMAT = 3,
    EBB_ERR_MESH = 4,
    EBB_ERR_CONFIG = 5,
    EBB_ERR_CUDA = 6,
    EBB_ERR_OOM = 7,
    EBB_ERR_NAN_EDGE = 8,   // replaces EdgeException (source/solve.d)
    EBB_ERR_NAN_CELL = 9,   // replaces CellException (app/solver.d:131-149)
    EBB_ERR_NO_DEVICE = 10,
    EBB_ERR_BC = 11,        // tpInflow without a non-negative Mach root (solve.d:662-669)
    EBB_ERR_LIMIT = 12
}

// ebb_bc_type: the order of enum BoundaryType (source/mesh.d:27-36)
enum : int
{
    EBB_BC_FULL_STATE = 0,
    EBB_BC_CONST_PRESSURE = 1,
    EBB_BC_INVISCID_WALL = 2,
    EBB_BC_VISCOUS_WALL = 3,
    EBB_BC_SYMMETRY = 4,
    EBB_BC_TEMP_PRES_INFLOW = 5,
    EBB_BC_DIRICHLET = 6
}

enum : int { EBB_FLUX_RUSANOV = 0, EBB_FLUX_ROE = 1 }                                  // fluxList
enum : int { EBB_INT_EULER = 0, EBB_INT_RK2 = 1, EBB_INT_RK2_TVD = 2, EBB_INT_RK4 = 3 } // integratorList
enum : int { EBB_PREC_FP64 = 0, EBB_PREC_SPLIT = 1, EBB_PREC_DF = 2 }
enum : int { EBB_MMS_NONE = 0, EBB_MMS_REFERENCE = 1, EBB_MMS_SINE = 2 }

struct ebb_boundary
{
    char[EBB_TAG_LEN] tag;
    int type;
    int n_data;
    double[8] data;
}

/// struct Config (source/config.d:72-94), flattened
struct ebb_config
{
    char[EBB_PATH_LEN] mesh_file;
    double dt;
    int dynamic_dt;
    double t_end;
    int flux;
    long save_iter;
    long plot_iter;
    int n_force;
    char[EBB_TAG_LEN][EBB_MAX_FORCE_TAGS] force_boundary;
    int integrator;
    int limited;
    double lp_thresh;
    long order;
    double cfl;
    double[4] ic;
    int n_boundaries;
    ebb_boundary[EBB_MAX_BC] boundaries;
    int local_timestep;
    int multistage_limiting;
    int cfl_adjust;
    int viscosity;
    double pr, r_gas, gamma, mu, re, l_ref;
    int mms;
}

struct ebb_mesh;
struct ebb_solver;
struct ebb_server;

struct ebb_mesh_info
{
    long n_nodes;
    long n_cells;
    long n_ghost;
    long n_edges;
    long n_int_edges;
    int n_tags;
    int max_edges;
    long face_slots;
}

/// one iteration of runIntegrator (app/solver.d:178-230)
struct ebb_step_record
{
    double t;
    double drag;
    double lift;
    double[4] resid;
    double rmax;
    double dt;
    double cfl;
}

struct ebb_instance_status
{
    long cell_offset;
    long n_cells;
    long iterations;
    double t, dt, cfl;
    int done;
    int status;
    long err_index;
    double drag, lift;
    double[4] resid;
    double rmax;
    double resid_first;
}

struct ebb_server_options
{
    int precision;
    int max_arenas;
    int max_batch;
    int build_threads;
    double tick_ms;
    double size_ratio;
    long arena_cells;
    ulong hbm_budget;
    int escalate;
    int finish_fp64;
    int stall_steps;
    int finish_precision;
}

struct ebb_request_result
{
    long id;
    int status;
    int done_reason;
    long err_index;
    long n_cells;
    long iterations;
    double t, drag, lift;
    double[4] resid;
    double resid_first;
    double submit_s, admit_s, finish_s;
    int precision;
    int escalated;
    long split_iterations;
    char[96] msg;
}

struct ebb_server_stats
{
    ulong bytes_in_use, bytes_peak;
    int arenas, waiting, building, reserved;
    long submitted, finished, cell_updates, escalations;
}

// ---- library
int ebb_abi_version();
int ebb_struct_sizes(size_t* config, size_t* mesh_info, size_t* step_record);
int ebb_device_count(int* n_devices);
int ebb_set_device(int device);
int ebb_host_alloc(size_t bytes, void** ptr);
int ebb_host_free(void* ptr);

// ---- config (source/config.d:112-313)
void ebb_config_defaults(ebb_config* cfg);
int ebb_config_parse(const(char)* json_text, ebb_config* out_, char* err, size_t err_len);

// ---- mesh (source/io.d:669-990, source/mesh.d:242-313)
int ebb_mesh_import(const(char)* path, ebb_mesh** out_, char* err, size_t err_len);
int ebb_mesh_from_arrays(long n_nodes, const(double)* xy, long n_elem, const(long)* elem_off,
                         const(int)* elem_nodes, long n_b, const(int)* b_nodes, int n_tags,
                         const(long)* b_group_start, const(char)* tags, ebb_mesh** out_, char* err,
                         size_t err_len);
int ebb_mesh_get_info(const(ebb_mesh)* mesh, ebb_mesh_info* info);
int ebb_mesh_get_tag(const(ebb_mesh)* mesh, int i, char* tag, size_t len);
int ebb_mesh_centroids(const(ebb_mesh)* mesh, double* xy);
int ebb_mesh_edges(const(ebb_mesh)* mesh, int* group, int* cells, double* mid, double* normal, double* len);
void ebb_mesh_free(ebb_mesh* mesh);

// ---- solver (buildMesh + ufvmSetup, ufvmSolver, integrators, runIntegrator)
int ebb_solver_create(const(ebb_mesh)* mesh, const(ebb_config)* cfg, int precision, ebb_solver** out_,
                      char* err, size_t err_len);
void ebb_solver_destroy(ebb_solver* s);
int ebb_last_error(const(ebb_solver)* s, int* kind, long* index, char* msg, size_t msg_len);
int ebb_set_state(ebb_solver* s, const(double)* q);
int ebb_get_state(ebb_solver* s, double* q);
int ebb_get_time(ebb_solver* s, double* t, double* dt, long* iterations);
int ebb_set_time(ebb_solver* s, double t, double dt);
int ebb_residual(ebb_solver* s, const(double)* q, double* R, double* new_dt, double* rmax, int limit,
                 int dt_update);
int ebb_residual_device(ebb_solver* s, const(double)* q_dev, double* R_dev, double* new_dt, double* rmax,
                        int limit, int dt_update);
int ebb_step(ebb_solver* s, double* dt, double* rmax);
int ebb_run(ebb_solver* s, long max_steps, ebb_step_record* records, long* steps_run);
int ebb_run_timed(ebb_solver* s, long max_steps, long* steps_run, double* device_ms);
int ebb_get_face_states(ebb_solver* s, double* out_);
int ebb_get_edge_fluxes(ebb_solver* s, double* out_);
int ebb_get_stream(ebb_solver* s, void** stream);
int ebb_profile_kernels(ebb_solver* s, int n_rep, double* ms);

// ---- batched arena (no counterpart in the reference)
int ebb_batch_create(int n, const(ebb_mesh*)* meshes, const(ebb_config)* cfgs, int precision,
                     ebb_solver** out_, char* err, size_t err_len);
int ebb_batch_size(const(ebb_solver)* s, int* n);
int ebb_batch_status(ebb_solver* s, int first, int count, ebb_instance_status* out_);
int ebb_batch_set_stop(ebb_solver* s, int k, double t_end, long max_steps, double resid_drop);
int ebb_batch_get_state(ebb_solver* s, int k, double* q);
int ebb_batch_set_state(ebb_solver* s, int k, const(double)* q);
int ebb_launch_steps(ebb_solver* s, long n_steps);
int ebb_sync(ebb_solver* s);
int ebb_batch_footprint(int n, const(ebb_mesh*)* meshes, const(ebb_config)* cfgs, int precision,
                        size_t* bytes, char* err, size_t err_len);

// ---- request server (no counterpart in the reference)
void ebb_server_options_defaults(ebb_server_options* o);
int ebb_server_create(const(ebb_server_options)* o, ebb_server** out_, char* err, size_t err_len);
int ebb_server_submit(ebb_server* sv, const(ebb_mesh)* mesh, const(ebb_config)* cfg, long max_steps,
                      double resid_drop, long* id);
int ebb_server_tick(ebb_server* sv, int* n_active, int* n_waiting);
int ebb_server_results(ebb_server* sv, ebb_request_result* out_, int cap, int* n);
int ebb_server_take_state(ebb_server* sv, long id, double* q);
int ebb_server_stats_get(ebb_server* sv, ebb_server_stats* st);
void ebb_server_destroy(ebb_server* sv);

// ---- flux seam (source/flux.d)
int ebb_flux(int kind, long n, const(double)* qL, const(double)* qR, const(double)* normal, double* F,
             double* s_max);
int ebb_flux_noalloc(int kind, long n, const(double)* qL, const(double)* qR, const(double)* normal, double* F,
                     double* s_max);

// ---- files (source/io.d) and ebb-reconstruct (app/reconstruct.d)
int ebb_save_solution(ebb_solver* s, const(char)* path, double t, double dt);
int ebb_load_solution(ebb_solver* s, const(char)* path);
int ebb_load_solution_parts(ebb_solver* s, int n, const(char*)* paths);
int ebb_reconstruct(ebb_solver* s, const(ebb_mesh)* mesh, const(char)* mmsh_path, const(char)* esln_path,
                    double t, double dt, double* q_out, long* n_out);

/// true when the library's struct sizes are this binding's
extern(D) bool checkLayout()
{
    size_t a, b, c;
    if (ebb_struct_sizes(&a, &b, &c) != EBB_OK)
        return false;
    return a == ebb_config.sizeof && b == ebb_mesh_info.sizeof && c == ebb_step_record.sizeof
        && ebb_abi_version() == EBB_ABI_VERSION;
}
