// solver.cpp -- solver handle: device layout build (buildMesh + ufvmSetup), stage
// scheduling of the integrators, the CUDA-graph time loop, and the C ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>

#include "solver_impl.hpp"

using namespace ebb;

namespace {


int cuda_status(cudaError_t e) { return e == cudaSuccess ? EBB_OK : (e == cudaErrorMemoryAllocation ? EBB_ERR_OOM : EBB_ERR_CUDA); }

int fail(ebb_solver *s, int code, const std::string &msg)
{
    if (s) {
        s->err_kind = code;
        s->err_msg = msg;
    }
    return code;
}

#define CK(x)                                                                                  \
    do {                                                                                       \
        cudaError_t _e = (x);                                                                  \
        if (_e != cudaSuccess) return fail(s, cuda_status(_e), std::string("CUDA: ") + cudaGetErrorString(_e)); \
    } while (0)
// Two CUDA events, destroyed on every return path of the function that holds them.
struct EventPair {
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t create()
    {
        cudaError_t e = cudaEventCreate(&ev[0]);
        return e == cudaSuccess ? cudaEventCreate(&ev[1]) : e;
    }
    ~EventPair()
    {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
};

#define CKL(x)                                                                                 \
    do {                                                                                       \
        int _r = (x);                                                                          \
        if (_r != 0) return fail(s, EBB_ERR_CUDA, "kernel launch failed");                     \
    } while (0)

// Page-locked buffers from ebb_host_alloc, by base address, with the address the
// device reads them at.  A state upload from inside one of them is read by the state
// kernel directly over the host link (in sequence; as fast as a copy engine on GB300,
// and it saves the staging copy's device pass).  Downloads always go through a
// staging array and a copy engine: device stores to host memory ran at less than
// half the copy engine's rate.
struct HostBuf {
    size_t bytes;
    char *dev;
};
std::mutex g_host_mu;
std::map<uintptr_t, HostBuf> g_host;

// device address of [p, p + bytes) when it lies inside one ebb_host_alloc buffer and
// starts on a 16-byte boundary (the state kernels move a cell as 16-byte vectors);
// otherwise null, and the caller stages through device memory
void *host_mapped(const void *p, size_t bytes)
{
    std::lock_guard<std::mutex> l(g_host_mu);
    const uintptr_t a = (uintptr_t)p;
    auto it = g_host.upper_bound(a);
    if (it == g_host.begin()) return nullptr;
    --it;
    if (a - it->first > it->second.bytes || bytes > it->second.bytes - (a - it->first)) return nullptr;
    char *d = it->second.dev + (a - it->first);
    return ((uintptr_t)d & 15u) == 0 ? d : nullptr;
}

// caller-order state (host) -> device state q64 (and its FP32 copy), cells [c0, c0+n)
int state_in(ebb_solver *s, const double *q, int64_t c0, int64_t n)
{
    const size_t nb = sizeof(double) * 4 * (size_t)n;
    const double *src = static_cast<const double *>(host_mapped(q, nb));
    if (!src) {
        CK(cudaMemcpyAsync(s->d_stage + 4 * c0, q, nb, cudaMemcpyHostToDevice, s->stream));
        src = s->d_stage + 4 * c0;
    }
    float *qs1 = s->precision == EBB_PREC_SPLIT ? reinterpret_cast<float *>(s->A.qs1) : nullptr;
    CKL(launch_load_state(src, s->A.q64, qs1, s->d_iperm + c0, n, s->stream));
    if (s->precision == EBB_PREC_DF) CKL(launch_to_df4(s->A.q64, s->A.qs1, s->C, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

// device state q64 -> caller-order state (host), cells [c0, c0+n)
int state_out(ebb_solver *s, double *q, int64_t c0, int64_t n)
{
    const size_t nb = sizeof(double) * 4 * (size_t)n;
    CKL(launch_store_state(s->A.q64, s->d_stage + 4 * c0, s->d_iperm + c0, n, s->stream));
    CK(cudaMemcpyAsync(q, s->d_stage + 4 * c0, nb, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

inline unsigned long long dbits(double v)
{
    unsigned long long u;
    std::memcpy(&u, &v, 8);
    return u;
}
inline double bitsd(unsigned long long u)
{
    double v;
    std::memcpy(&v, &u, 8);
    return v;
}

template <typename T>
int run_stage_t(ebb_solver *s, int stage, T *qin, T *qout, int limit, int dt_update, int need_dt, int final_stage)
{
    CKL(launch_cell<T>(s->M, s->P, s->A, qin, limit, s->stream));
    CKL(launch_flux<T>(s->M, s->P, s->A, qin, s->stream));
    CKL(launch_update<T>(s->M, s->P, s->A, stage, qin, qout, dt_update, need_dt, final_stage, s->stream));
    return EBB_OK;
}

// integrators.d: stage sequence of one step on the resident state
template <typename T> int integrator_stages_t(ebb_solver *s)
{
    const ebb_config &c = s->cfg;
    T *q1 = reinterpret_cast<T *>(s->A.qs1), *qs = reinterpret_cast<T *>(s->A.qs);
    const int ms = c.multistage_limiting;
    const int lts = c.local_timestep;
    int r = EBB_OK;
    switch (c.integrator) {
    case EBB_INT_EULER:
        r = run_stage_t<T>(s, ST_EULER, q1, q1, 1, 1, 1, 1);
        break;
    case EBB_INT_RK2:
        if ((r = run_stage_t<T>(s, ST_RK2_1, q1, qs, 1, 1, 0, 0))) break;
        r = run_stage_t<T>(s, ST_RK2_2, qs, q1, ms, 0, 1, 1);
        break;
    case EBB_INT_RK2_TVD:
        if ((r = run_stage_t<T>(s, ST_TVD_1, q1, qs, 1, lts, 0, 0))) break;
        r = run_stage_t<T>(s, ST_TVD_2, qs, q1, 0, !lts, 1, 1);
        break;
    case EBB_INT_RK4:
        if ((r = run_stage_t<T>(s, ST_RK4_1, q1, qs, 1, 1, 0, 0))) break;
        if ((r = run_stage_t<T>(s, ST_RK4_2, qs, qs, ms, 0, 0, 0))) break;
        if ((r = run_stage_t<T>(s, ST_RK4_3, qs, qs, ms, 0, 0, 0))) break;
        r = run_stage_t<T>(s, ST_RK4_4, qs, q1, ms, 0, 1, 1);
        break;
    default:
        r = fail(s, EBB_ERR_CONFIG, "unknown integrator");
    }
    return r;
}

int integrator_stages(ebb_solver *s)
{
    if (s->precision == EBB_PREC_SPLIT) return integrator_stages_t<float>(s);
    if (s->precision == EBB_PREC_DF) return integrator_stages_t<ebbdf::df>(s);
    return integrator_stages_t<double>(s);
}

int one_loop_step(ebb_solver *s)
{
    int r = integrator_stages(s);
    if (r) return r;
    CKL(launch_step_end(s->M, s->A, s->nred, s->precision, s->stream));
    return EBB_OK;
}

// stage kernels of one residual evaluation on the stage buffer qs (ST_RESID writes R)
int residual_kernels(ebb_solver *s, int limit, int dt_update)
{
    if (s->precision == EBB_PREC_SPLIT) {
        float *qs = reinterpret_cast<float *>(s->A.qs);
        return run_stage_t<float>(s, ST_RESID, qs, nullptr, limit, dt_update, 1, 0);
    }
    if (s->precision == EBB_PREC_DF) {
        ebbdf::df *qs = reinterpret_cast<ebbdf::df *>(s->A.qs);
        return run_stage_t<ebbdf::df>(s, ST_RESID, qs, nullptr, limit, dt_update, 1, 0);
    }
    double *qs = reinterpret_cast<double *>(s->A.qs);
    return run_stage_t<double>(s, ST_RESID, qs, nullptr, limit, dt_update, 1, 0);
}

int build_graph(ebb_solver *s, int steps, cudaGraphExec_t *out)
{
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int r = EBB_OK;
    for (int k = 0; k < steps && r == EBB_OK; k++) r = one_loop_step(s);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (r) return r;
    CK(e);
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    return EBB_OK;
}

int ensure_graphs(ebb_solver *s)
{
    int r;
    if (!s->g1 && (r = build_graph(s, 1, &s->g1))) return r;
    if (!s->g16 && (r = build_graph(s, 16, &s->g16))) return r;
    return EBB_OK;
}

int enqueue_steps(ebb_solver *s, int64_t n)
{
    int64_t k = 0;
    for (; k + 16 <= n; k += 16) CK(cudaGraphLaunch(s->g16, s->stream));
    for (; k < n; k++) CK(cudaGraphLaunch(s->g1, s->stream));
    return EBB_OK;
}

bool all_done(const std::vector<DState> &h)
{
    for (const DState &x : h)
        if (!x.done) return false;
    return true;
}

int decode_error(ebb_solver *s, const DState &h)
{
    if (h.err_key == EBB_NOERR) return EBB_OK;
    int code = (int)((h.err_key >> 40) & 0xff);
    s->err_kind = code;
    s->err_index = (int64_t)(h.err_key & 0xffffffffffull);
    switch (code) {
    case 8: s->err_msg = "Got NaN on edge flux"; break;
    case 9: s->err_msg = "Got nan on cell average value"; break;
    case 11: s->err_msg = "Both computed mach numbers are negative"; break;
    default: s->err_msg = "solver error";
    }
    return code;
}

}  // namespace

namespace ebb {

int solver_sync_state(ebb_solver *s, DState &h)
{
    CK(cudaMemcpyAsync(&h, s->A.st, sizeof(DState), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

int solver_write_state(ebb_solver *s, const DState &h)
{
    CK(cudaMemcpyAsync(s->A.st, &h, sizeof(DState), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

int solver_sync_all(ebb_solver *s, std::vector<DState> &h)
{
    h.resize(s->n_inst);
    CK(cudaMemcpyAsync(h.data(), s->A.st, sizeof(DState) * s->n_inst, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

int solver_write_all(ebb_solver *s, const std::vector<DState> &h)
{
    CK(cudaMemcpyAsync(s->A.st, h.data(), sizeof(DState) * s->n_inst, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

}  // namespace ebb

template <typename T> int profile_t(ebb_solver *s, int32_t n_rep, double *ms)
{
    // work on a copy of the stage-1 state so the resident solution is untouched
    const size_t bytes = sizeof(T) * 4 * (size_t)(s->C + s->G);
    CK(cudaMemcpyAsync(s->A.qs, s->A.qs1, bytes, cudaMemcpyDeviceToDevice, s->stream));
    T *qs = reinterpret_cast<T *>(s->A.qs);
    T *scratch = reinterpret_cast<T *>(s->A.face);  // update output target (rebuilt below)
    EventPair evp;
    CK(evp.create());
    cudaEvent_t *ev = evp.ev;
    for (int k = 0; k < 4; k++) {
        float t = 0;
        CK(cudaEventRecord(ev[0], s->stream));
        for (int i = 0; i < n_rep; i++) {
            if (k == 0) CKL(launch_cell<T>(s->M, s->P, s->A, qs, 1, s->stream));
            if (k == 1) CKL(launch_flux<T>(s->M, s->P, s->A, qs, s->stream));
            if (k == 2) CKL(launch_update<T>(s->M, s->P, s->A, ST_RK2_1, qs, scratch, 1, 1, 0, s->stream));
            if (k == 3) CKL(launch_step_end(s->M, s->A, s->nred, s->precision, s->stream));
        }
        CK(cudaEventRecord(ev[1], s->stream));
        CK(cudaEventSynchronize(ev[1]));
        CK(cudaEventElapsedTime(&t, ev[0], ev[1]));
        ms[k] = (double)t / n_rep;
        if (k == 2) CKL(launch_cell<T>(s->M, s->P, s->A, qs, 1, s->stream));
    }
    return EBB_OK;
}

extern "C" {

int ebb_abi_version(void) { return EBB_ABI_VERSION; }

int ebb_struct_sizes(size_t *config, size_t *mesh_info, size_t *step_record)
{
    if (config) *config = sizeof(ebb_config);
    if (mesh_info) *mesh_info = sizeof(ebb_mesh_info);
    if (step_record) *step_record = sizeof(ebb_step_record);
    return EBB_OK;
}

int ebb_device_count(int *n)
{
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (n) *n = (e == cudaSuccess) ? c : 0;
    return (e == cudaSuccess && c > 0) ? EBB_OK : EBB_ERR_NO_DEVICE;
}

int ebb_set_device(int device)
{
    return cudaSetDevice(device) == cudaSuccess ? EBB_OK : EBB_ERR_NO_DEVICE;
}

int ebb_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr) return EBB_ERR_ARG;
    if (cudaMallocHost(ptr, bytes) != cudaSuccess) return EBB_ERR_OOM;
    void *dev = nullptr;
    if (cudaHostGetDevicePointer(&dev, *ptr, 0) == cudaSuccess && dev) {
        std::lock_guard<std::mutex> l(g_host_mu);
        g_host[(uintptr_t)*ptr] = HostBuf{bytes, static_cast<char *>(dev)};
    } else {
        cudaGetLastError();  // not device-mapped: state copies stage through device memory
    }
    return EBB_OK;
}

int ebb_host_free(void *ptr)
{
    {
        std::lock_guard<std::mutex> l(g_host_mu);
        g_host.erase((uintptr_t)ptr);
    }
    return cudaFreeHost(ptr) == cudaSuccess ? EBB_OK : EBB_ERR_CUDA;
}

int ebb_solver_create(const ebb_mesh *mesh, const ebb_config *cfg, int32_t precision, ebb_solver **out, char *err,
                      size_t err_len)
{
    if (!mesh || !cfg || !out) return EBB_ERR_ARG;
    return ebb_batch_create(1, &mesh, cfg, precision, out, err, err_len);
}

int ebb_batch_create(int32_t n, const ebb_mesh *const *meshes, const ebb_config *cfgs, int32_t precision,
                     ebb_solver **out, char *err, size_t err_len)
{
    if (!out) return EBB_ERR_ARG;
    *out = nullptr;
    if (n <= 0 || !meshes || !cfgs) return EBB_ERR_ARG;
    for (int32_t k = 0; k < n; k++)
        if (!meshes[k]) return EBB_ERR_ARG;
    if (precision != EBB_PREC_FP64 && precision != EBB_PREC_SPLIT && precision != EBB_PREC_DF) {
        set_err(err, err_len, "unknown precision form");
        return EBB_ERR_ARG;
    }
    int ndev = 0;
    if (ebb_device_count(&ndev) != EBB_OK) {
        set_err(err, err_len, "no CUDA device available");
        return EBB_ERR_NO_DEVICE;
    }
    // host layouts of the instances, built in parallel (independent meshes)
    std::vector<InstLayout> Ls(n);
    std::vector<int> rc(n, EBB_OK);
    std::vector<std::string> msg(n);
    const int nt = (int)std::min<unsigned>((unsigned)n, std::max(1u, std::thread::hardware_concurrency()));
    auto work = [&](int t0) {
        for (int32_t k = t0; k < n; k += nt) rc[k] = build_instance(meshes[k], &cfgs[k], Ls[k], msg[k]);
    };
    if (nt == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++) th.emplace_back(work, t);
        for (auto &x : th) x.join();
    }
    for (int32_t k = 0; k < n; k++)
        if (rc[k]) {
            set_err(err, err_len, n > 1 ? "instance " + std::to_string(k) + ": " + msg[k] : msg[k]);
            return rc[k];
        }
    std::string e;
    auto *s = new ebb_solver();
    int r = assemble(s, Ls, precision, e);
    if (r) {
        set_err(err, err_len, e);
        ebb_solver_destroy(s);
        return r;
    }
    *out = s;
    return EBB_OK;
}

void ebb_solver_destroy(ebb_solver *s)
{
    if (!s) return;
    if (s->g1) cudaGraphExecDestroy(s->g1);
    if (s->g16) cudaGraphExecDestroy(s->g16);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->dmem) cudaFree(s->dmem);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int ebb_last_error(const ebb_solver *s, int32_t *kind, int64_t *index, char *msg, size_t msg_len)
{
    if (!s) return EBB_ERR_ARG;
    if (kind) *kind = s->err_kind;
    if (index) *index = s->err_index;
    set_err(msg, msg_len, s->err_msg);
    return EBB_OK;
}

int ebb_set_state(ebb_solver *s, const double *q)
{
    if (!s || !q) return EBB_ERR_ARG;
    return state_in(s, q, 0, s->C);
}

int ebb_get_state(ebb_solver *s, double *q)
{
    if (!s || !q) return EBB_ERR_ARG;
    return state_out(s, q, 0, s->C);
}

int ebb_get_time(ebb_solver *s, double *t, double *dt, int64_t *iterations)
{
    if (!s) return EBB_ERR_ARG;
    DState h;
    int r = solver_sync_state(s, h);
    if (r) return r;
    if (t) *t = h.t;
    if (dt) *dt = h.dt;
    if (iterations) *iterations = h.iter;
    return EBB_OK;
}

int ebb_set_time(ebb_solver *s, double t, double dt)
{
    if (!s) return EBB_ERR_ARG;
    DState h;
    int r = solver_sync_state(s, h);
    if (r) return r;
    h.t = t;
    set_step(h, dt);
    h.done = !(h.t < h.t_end);
    return solver_write_state(s, h);
}

int ebb_residual(ebb_solver *s, const double *q, double *R, double *new_dt, double *rmax, int32_t limit,
                 int32_t dt_update)
{
    if (!s || !q || !R) return EBB_ERR_ARG;
    if (s->n_inst != 1) return fail(s, EBB_ERR_ARG, "not available on a batch of several instances");
    CK(cudaMemcpyAsync(s->d_stage, q, sizeof(double) * 4 * s->C, cudaMemcpyHostToDevice, s->stream));
    int r = ebb_residual_device(s, s->d_stage, s->d_stage, new_dt, rmax, limit, dt_update);
    if (r) return r;
    CK(cudaMemcpyAsync(R, s->d_stage, sizeof(double) * 4 * s->C, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

int ebb_residual_device(ebb_solver *s, const double *q_dev, double *R_dev, double *new_dt, double *rmax, int32_t limit,
                        int32_t dt_update)
{
    if (!s || !q_dev || !R_dev) return EBB_ERR_ARG;
    if (s->n_inst != 1) return fail(s, EBB_ERR_ARG, "not available on a batch of several instances");
    const bool split = s->precision == EBB_PREC_SPLIT, dfp = s->precision == EBB_PREC_DF;
    if (split) {
        CKL(launch_permute4(q_dev, s->d_tmp, s->d_perm, s->C, 1, s->stream));
        CKL(launch_to_float4(s->d_tmp, reinterpret_cast<float *>(s->A.qs), s->C, s->stream));
    } else if (dfp) {
        CKL(launch_permute4(q_dev, s->d_tmp, s->d_perm, s->C, 1, s->stream));
        CKL(launch_to_df4(s->d_tmp, s->A.qs, s->C, s->stream));
    } else {
        CKL(launch_permute4(q_dev, reinterpret_cast<double *>(s->A.qs), s->d_perm, s->C, 1, s->stream));
    }
    int r = solver_run_residual_on_qs(s, limit, dt_update, new_dt, rmax);
    if (r) return r;
    if (split) {
        CKL(launch_to_double4(reinterpret_cast<const float *>(s->A.R), s->d_tmp, s->C, s->stream));
        CKL(launch_permute4(s->d_tmp, R_dev, s->d_perm, s->C, 0, s->stream));
    } else if (dfp) {
        CKL(launch_from_df4(s->A.R, s->d_tmp, s->C, s->stream));
        CKL(launch_permute4(s->d_tmp, R_dev, s->d_perm, s->C, 0, s->stream));
    } else {
        CKL(launch_permute4(reinterpret_cast<const double *>(s->A.R), R_dev, s->d_perm, s->C, 0, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

int ebb_step(ebb_solver *s, double *dt, double *rmax)
{
    if (!s || !dt || !rmax) return EBB_ERR_ARG;
    if (s->n_inst != 1) return fail(s, EBB_ERR_ARG, "not available on a batch of several instances");
    DState h;
    int r = solver_sync_state(s, h);
    if (r) return r;
    const int saved_done = h.done;
    set_step(h, *dt);
    h.newdt_bits = 0x7FF0000000000000ull;
    h.rmax_bits = (*rmax > 0) ? dbits(*rmax) : 0ull;
    h.done = 0;
    if ((r = solver_write_state(s, h))) return r;
    if ((r = integrator_stages(s))) return r;
    if ((r = solver_sync_state(s, h))) return r;
    *dt = bitsd(h.newdt_bits);
    *rmax = bitsd(h.rmax_bits);
    h.done = saved_done;
    int code = decode_error(s, h);
    h.err_key = EBB_NOERR;
    if ((r = solver_write_state(s, h))) return r;
    return code;
}

int ebb_run(ebb_solver *s, int64_t max_steps, ebb_step_record *records, int64_t *steps_run)
{
    if (!s || max_steps < 0) return EBB_ERR_ARG;
    if (steps_run) *steps_run = 0;
    const bool single = s->n_inst == 1;
    std::vector<DState> h;
    int r = solver_sync_all(s, h);
    if (r) return r;
    if (single && h[0].err_key != EBB_NOERR) return decode_error(s, h[0]);
    if (all_done(h)) return EBB_OK;
    if ((r = ensure_graphs(s))) return r;
    int64_t run = 0;
    std::vector<int64_t> it0(s->n_inst);
    while (run < max_steps) {
        const int64_t chunk = std::min<int64_t>(max_steps - run, EBB_REC_CAP);
        for (int k = 0; k < s->n_inst; k++) it0[k] = h[k].iter;
        const int64_t rec0 = h[0].n_rec;
        if ((r = enqueue_steps(s, chunk))) return r;
        if ((r = solver_sync_all(s, h))) return r;
        int64_t did = 0;
        for (int k = 0; k < s->n_inst; k++) did = std::max<int64_t>(did, h[k].iter - it0[k]);
        if (single && records && h[0].n_rec > rec0) {
            for (int64_t m = rec0; m < h[0].n_rec; m++) {
                CK(cudaMemcpyAsync(&records[run + (m - rec0)], &s->A.rec[m % EBB_REC_CAP], sizeof(DRecord),
                                   cudaMemcpyDeviceToHost, s->stream));
            }
            CK(cudaStreamSynchronize(s->stream));
        }
        run += did;
        if (single && h[0].err_key != EBB_NOERR) {
            if (steps_run) *steps_run = run;
            return decode_error(s, h[0]);
        }
        if (all_done(h) || did < chunk) break;
    }
    if (steps_run) *steps_run = run;
    return EBB_OK;
}

int ebb_run_timed(ebb_solver *s, int64_t max_steps, int64_t *steps_run, double *device_ms)
{
    if (!s || max_steps < 0 || !device_ms) return EBB_ERR_ARG;
    if (steps_run) *steps_run = 0;
    *device_ms = 0;
    std::vector<DState> h;
    int r = solver_sync_all(s, h);
    if (r) return r;
    if (s->n_inst == 1 && h[0].err_key != EBB_NOERR) return decode_error(s, h[0]);
    if ((r = ensure_graphs(s))) return r;
    std::vector<int64_t> it0(s->n_inst);
    for (int k = 0; k < s->n_inst; k++) it0[k] = h[k].iter;
    EventPair evp;
    CK(evp.create());
    cudaEvent_t *ev = evp.ev;
    CK(cudaEventRecord(ev[0], s->stream));
    if ((r = enqueue_steps(s, max_steps))) return r;
    CK(cudaEventRecord(ev[1], s->stream));
    CK(cudaEventSynchronize(ev[1]));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    *device_ms = ms;
    if ((r = solver_sync_all(s, h))) return r;
    int64_t did = 0;
    for (int k = 0; k < s->n_inst; k++) did = std::max<int64_t>(did, h[k].iter - it0[k]);
    if (steps_run) *steps_run = did;
    return s->n_inst == 1 ? decode_error(s, h[0]) : EBB_OK;
}

int ebb_get_stream(ebb_solver *s, void **stream)
{
    if (!s || !stream) return EBB_ERR_ARG;
    *stream = (void *)s->stream;
    return EBB_OK;
}

int ebb_profile_kernels(ebb_solver *s, int32_t n_rep, double *ms)
{
    if (!s || !ms || n_rep <= 0) return EBB_ERR_ARG;
    std::vector<DState> h0;
    int r = solver_sync_all(s, h0);
    if (r) return r;
    std::vector<DState> h = h0;
    for (DState &x : h) {
        x.done = 0;
        x.err_key = EBB_NOERR;
        x.rec_enabled = 0;
    }
    if ((r = solver_write_all(s, h))) return r;
    r = s->precision == EBB_PREC_SPLIT ? profile_t<float>(s, n_rep, ms)
        : s->precision == EBB_PREC_DF  ? profile_t<ebbdf::df>(s, n_rep, ms)
                                       : profile_t<double>(s, n_rep, ms);
    int r2 = solver_write_all(s, h0);
    return r ? r : r2;
}

int ebb_get_face_states(ebb_solver *s, double *out)
{
    if (!s || !out) return EBB_ERR_ARG;
    const size_t n = 4 * (size_t)s->maxJ * s->Cs;
    std::vector<double> f(n);
    if (s->precision == EBB_PREC_SPLIT) {
        std::vector<float> g(n);
        CK(cudaMemcpyAsync(g.data(), s->A.face, n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (size_t k = 0; k < n; k++) f[k] = g[k];
    } else if (s->precision == EBB_PREC_DF) {
        std::vector<ebbdf::df> g(n);
        CK(cudaMemcpyAsync(g.data(), s->A.face, n * sizeof(ebbdf::df), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (size_t k = 0; k < n; k++) f[k] = (double)g[k];
    } else {
        CK(cudaMemcpyAsync(f.data(), s->A.face, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    for (size_t k = 0; k < s->ref_face_slot.size(); k++)
        for (int c = 0; c < 4; c++) out[4 * k + c] = f[4 * s->ref_face_slot[k] + c];
    return EBB_OK;
}

int ebb_get_edge_fluxes(ebb_solver *s, double *out)
{
    if (!s || !out || s->n_inst != 1) return EBB_ERR_ARG;
    const size_t n = 4 * (size_t)(s->Eint + s->G);
    std::vector<double> f(n);
    if (s->precision == EBB_PREC_SPLIT) {
        std::vector<float> g(n);
        CK(cudaMemcpyAsync(g.data(), s->A.fl, n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (size_t k = 0; k < n; k++) f[k] = g[k];
    } else if (s->precision == EBB_PREC_DF) {
        std::vector<ebbdf::df> g(n);
        CK(cudaMemcpyAsync(g.data(), s->A.fl, n * sizeof(ebbdf::df), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (size_t k = 0; k < n; k++) f[k] = (double)g[k];
    } else {
        CK(cudaMemcpyAsync(f.data(), s->A.fl, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    for (size_t e = 0; e < s->flux_ref.size(); e++)
        for (int c = 0; c < 4; c++) out[4 * (size_t)s->flux_ref[e] + c] = f[4 * e + c];
    return EBB_OK;
}

int ebb_flux(int32_t kind, int64_t n, const double *qL, const double *qR, const double *normal, double *F, double *s_max)
{
    if (n < 0 || (n && (!qL || !qR || !normal || !F || !s_max))) return EBB_ERR_ARG;
    if (n == 0) return EBB_OK;
    ebb_solver *s = nullptr;
    int nd = 0;
    if (ebb_device_count(&nd) != EBB_OK) return EBB_ERR_NO_DEVICE;
    double *d = nullptr;
    size_t tot = (size_t)n * (4 + 4 + 2 + 4 + 1);
    CK(cudaMalloc(&d, tot * sizeof(double)));
    double *dL = d, *dR = d + 4 * n, *dn = d + 8 * n, *dF = d + 10 * n, *ds = d + 14 * n;
    // the kernel runs only on inputs that arrived: the first failed upload ends the call
    cudaError_t e = cudaMemcpy(dL, qL, sizeof(double) * 4 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dR, qR, sizeof(double) * 4 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dn, normal, sizeof(double) * 2 * n, cudaMemcpyHostToDevice);
    int r = e == cudaSuccess ? launch_flux_batch(kind, n, dL, dR, dn, dF, ds, nullptr) : 0;
    if (e == cudaSuccess && !r) e = cudaMemcpy(F, dF, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && !r) e = cudaMemcpy(s_max, ds, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (r || e != cudaSuccess) return EBB_ERR_CUDA;
    return EBB_OK;
}

int ebb_batch_size(const ebb_solver *s, int32_t *n)
{
    if (!s || !n) return EBB_ERR_ARG;
    *n = s->n_inst;
    return EBB_OK;
}

int ebb_batch_status(ebb_solver *s, int32_t first, int32_t count, ebb_instance_status *out)
{
    if (!s || !out || first < 0 || count < 0 || first + (int64_t)count > s->n_inst) return EBB_ERR_ARG;
    if (count == 0) return EBB_OK;
    std::vector<DState> h(count);
    CK(cudaMemcpyAsync(h.data(), s->A.st + first, sizeof(DState) * count, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    for (int32_t j = 0; j < count; j++) {
        const DState &x = h[j];
        const InstMeta &m = s->inst[first + j];
        ebb_instance_status &o = out[j];
        std::memset(&o, 0, sizeof o);
        o.cell_offset = m.c0;
        o.n_cells = m.C;
        o.iterations = x.iter;
        o.t = x.t;
        o.dt = x.dt;
        o.cfl = x.cfl;
        o.done = x.done;
        o.status = x.err_key == EBB_NOERR ? EBB_OK : (int32_t)((x.err_key >> 40) & 0xff);
        o.err_index = x.err_key == EBB_NOERR ? -1 : (int64_t)(x.err_key & 0xffffffffffull);
        o.drag = x.last[0];
        o.lift = x.last[1];
        for (int k = 0; k < 4; k++) o.resid[k] = x.last[2 + k];
        o.rmax = x.last[6];
        o.resid_first = x.resid_first;
    }
    return EBB_OK;
}

int ebb_batch_set_stop(ebb_solver *s, int32_t k, double t_end, int64_t max_steps, double resid_drop)
{
    if (!s || k >= s->n_inst) return EBB_ERR_ARG;
    std::vector<DState> h;
    int r = solver_sync_all(s, h);
    if (r) return r;
    for (int32_t j = 0; j < s->n_inst; j++) {
        if (k >= 0 && j != k) continue;
        DState &x = h[j];
        x.t_end = t_end;
        x.max_steps = max_steps;
        x.stop_drop = resid_drop;
        x.done = x.err_key != EBB_NOERR || !(x.t < x.t_end) || (max_steps > 0 && x.iter >= max_steps);
    }
    return solver_write_all(s, h);
}

int ebb_batch_get_state(ebb_solver *s, int32_t k, double *q)
{
    if (!s || !q || k < 0 || k >= s->n_inst) return EBB_ERR_ARG;
    const InstMeta &m = s->inst[k];
    return state_out(s, q, m.c0, m.C);
}

int ebb_batch_set_state(ebb_solver *s, int32_t k, const double *q)
{
    if (!s || !q || k < 0 || k >= s->n_inst) return EBB_ERR_ARG;
    const InstMeta &m = s->inst[k];
    return state_in(s, q, m.c0, m.C);
}

int ebb_launch_steps(ebb_solver *s, int64_t n_steps)
{
    if (!s || n_steps < 0) return EBB_ERR_ARG;
    int r = ensure_graphs(s);
    if (r) return r;
    return enqueue_steps(s, n_steps);
}

int ebb_sync(ebb_solver *s)
{
    if (!s) return EBB_ERR_ARG;
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

int ebb_batch_footprint(int32_t n, const ebb_mesh *const *meshes, const ebb_config *cfgs, int32_t precision,
                        size_t *bytes, char *err, size_t err_len)
{
    if (n <= 0 || !meshes || !cfgs || !bytes) return EBB_ERR_ARG;
    std::vector<InstLayout> Ls(n);
    std::string e;
    for (int32_t k = 0; k < n; k++) {
        if (!meshes[k]) return EBB_ERR_ARG;
        int r = build_instance(meshes[k], &cfgs[k], Ls[k], e);
        if (r) {
            set_err(err, err_len, e);
            return r;
        }
    }
    *bytes = arena_bytes(Ls, precision);
    return EBB_OK;
}

}  // extern "C"

namespace ebb {

int solver_run_residual_on_qs(ebb_solver *s, int limit, int dt_update, double *new_dt, double *rmax)
{
    DState h;
    int r = solver_sync_state(s, h);
    if (r) return r;
    const int saved_done = h.done;
    h.newdt_bits = 0x7FF0000000000000ull;
    h.rmax_bits = (rmax && *rmax > 0) ? dbits(*rmax) : 0ull;
    h.done = 0;
    h.err_key = EBB_NOERR;
    if ((r = solver_write_state(s, h))) return r;
    if ((r = residual_kernels(s, limit, dt_update))) return r;
    if ((r = solver_sync_state(s, h))) return r;
    if (new_dt) *new_dt = bitsd(h.newdt_bits);
    if (rmax) *rmax = bitsd(h.rmax_bits);
    int code = decode_error(s, h);
    h.done = saved_done;
    h.err_key = EBB_NOERR;
    h.newdt_bits = 0x7FF0000000000000ull;
    h.rmax_bits = 0;
    if ((r = solver_write_state(s, h))) return r;
    return code;
}

}  // namespace ebb
