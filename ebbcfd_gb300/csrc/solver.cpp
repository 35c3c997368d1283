// solver.cpp -- solver handle: device layout build (buildMesh + ufvmSetup), stage
// scheduling of the integrators, the CUDA-graph time loop, and the C ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "solver_impl.hpp"

using namespace ebb;

namespace {

constexpr int K = kMaxEdges;

struct Arena {
    char *base = nullptr;
    size_t off = 0, cap = 0;
    template <typename T> T *take(size_t n)
    {
        size_t bytes = ((n * sizeof(T)) + 255) & ~(size_t)255;
        T *p = reinterpret_cast<T *>(base + off);
        off += bytes;
        return p;
    }
};

template <typename T> size_t sz(size_t n) { return ((n * sizeof(T)) + 255) & ~(size_t)255; }

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
#define CKL(x)                                                                                 \
    do {                                                                                       \
        int _r = (x);                                                                          \
        if (_r != 0) return fail(s, EBB_ERR_CUDA, "kernel launch failed");                     \
    } while (0)

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

void freestream(double M, double aoa_deg, double rho, double q[4])
{
    // solve.d:177-202 (U = 1, a = U/M, p = rho a^2 / gamma)
    double aoa = aoa_deg * (M_PI / 180);
    double U = 1.0, a = U / M, p = (rho * (a * a)) / 1.4, u = U * std::cos(aoa), v = U * std::sin(aoa);
    q[0] = rho;
    q[1] = rho * u;
    q[2] = rho * v;
    q[3] = p / (1.4 - 1.0) + 0.5 * rho * (u * u + v * v);
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
    return s->precision == EBB_PREC_SPLIT ? integrator_stages_t<float>(s) : integrator_stages_t<double>(s);
}

int one_loop_step(ebb_solver *s)
{
    int r = integrator_stages(s);
    if (r) return r;
    CKL(launch_step_end(s->M, s->A, s->nred, s->precision == EBB_PREC_SPLIT, s->stream));
    return EBB_OK;
}

// stage kernels of one residual evaluation on the stage buffer qs (ST_RESID writes R)
int residual_kernels(ebb_solver *s, int limit, int dt_update)
{
    if (s->precision == EBB_PREC_SPLIT) {
        float *qs = reinterpret_cast<float *>(s->A.qs);
        return run_stage_t<float>(s, ST_RESID, qs, nullptr, limit, dt_update, 1, 0);
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

}  // namespace ebb

template <typename T> int profile_t(ebb_solver *s, int32_t n_rep, double *ms)
{
    // work on a copy of the stage-1 state so the resident solution is untouched
    const size_t bytes = sizeof(T) * 4 * (size_t)(s->C + s->G);
    CK(cudaMemcpyAsync(s->A.qs, s->A.qs1, bytes, cudaMemcpyDeviceToDevice, s->stream));
    T *qs = reinterpret_cast<T *>(s->A.qs);
    T *scratch = reinterpret_cast<T *>(s->A.face);  // update output target (rebuilt below)
    cudaEvent_t ev[2];
    CK(cudaEventCreate(&ev[0]));
    CK(cudaEventCreate(&ev[1]));
    for (int k = 0; k < 4; k++) {
        float t = 0;
        CK(cudaEventRecord(ev[0], s->stream));
        for (int i = 0; i < n_rep; i++) {
            if (k == 0) CKL(launch_cell<T>(s->M, s->P, s->A, qs, 1, s->stream));
            if (k == 1) CKL(launch_flux<T>(s->M, s->P, s->A, qs, s->stream));
            if (k == 2) CKL(launch_update<T>(s->M, s->P, s->A, ST_RK2_1, qs, scratch, 1, 1, 0, s->stream));
            if (k == 3) CKL(launch_step_end(s->M, s->A, s->nred, sizeof(T) == 4, s->stream));
        }
        CK(cudaEventRecord(ev[1], s->stream));
        CK(cudaEventSynchronize(ev[1]));
        CK(cudaEventElapsedTime(&t, ev[0], ev[1]));
        ms[k] = (double)t / n_rep;
        if (k == 2) CKL(launch_cell<T>(s->M, s->P, s->A, qs, 1, s->stream));
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
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
    return cudaMallocHost(ptr, bytes) == cudaSuccess ? EBB_OK : EBB_ERR_OOM;
}

int ebb_host_free(void *ptr) { return cudaFreeHost(ptr) == cudaSuccess ? EBB_OK : EBB_ERR_CUDA; }

int ebb_solver_create(const ebb_mesh *mesh, const ebb_config *cfg, int32_t precision, ebb_solver **out, char *err,
                      size_t err_len)
{
    if (!mesh || !cfg || !out) return EBB_ERR_ARG;
    *out = nullptr;
    if (precision != EBB_PREC_FP64 && precision != EBB_PREC_SPLIT) {
        set_err(err, err_len, "unknown precision form");
        return EBB_ERR_ARG;
    }
    int ndev = 0;
    if (ebb_device_count(&ndev) != EBB_OK) {
        set_err(err, err_len, "no CUDA device available");
        return EBB_ERR_NO_DEVICE;
    }
    Topology t;
    std::string e;
    if (!build_topology(*mesh, t, e)) {
        set_err(err, err_len, e);
        return EBB_ERR_MESH;
    }
    // BC binding by tag (solve.d:222-278)
    const int nG = (int)mesh->tags.size();
    std::vector<int> group_bc(nG, -1);
    for (int g = 0; g < nG; g++) {
        for (int b = 0; b < cfg->n_boundaries; b++)
            if (mesh->tags[g] == cfg->boundaries[b].tag) {
                group_bc[g] = b;
                break;
            }
        if (group_bc[g] < 0) {
            set_err(err, err_len, "Could not find matching boundary condition tag " + mesh->tags[g]);
            return EBB_ERR_CONFIG;
        }
        const ebb_boundary &B = cfg->boundaries[group_bc[g]];
        if (B.type == EBB_BC_CONST_PRESSURE && B.n_data != 1) {
            set_err(err, err_len, "Constant pressure boundary data should only have one element; the constant pressure");
            return EBB_ERR_CONFIG;
        }
        if (B.type == EBB_BC_TEMP_PRES_INFLOW && B.n_data != 3) {
            set_err(err, err_len, "Constant temperature/pressure/aoa boundary data should have three elements");
            return EBB_ERR_CONFIG;
        }
        if (B.type == EBB_BC_FULL_STATE && B.n_data < 4) {
            set_err(err, err_len, "fullState boundary data needs [M, aoa, p, rho]");
            return EBB_ERR_CONFIG;
        }
    }

    auto *s = new ebb_solver();
    s->cfg = *cfg;
    s->precision = precision;
    const int64_t C = t.C, G = t.G;
    s->C = C;
    s->G = G;
    s->maxJ = t.maxJ;
    s->Cs = (C + 31) & ~(int64_t)31;
    const int64_t Cs = s->Cs;
    const int MJ = t.maxJ;
    s->mu = cfg->viscosity ? (cfg->ic[3] * 1.0 * cfg->l_ref) / cfg->re : NAN;

    // ---- orderings ----------------------------------------------------------
    s->perm = rcm_order(t);
    std::vector<int32_t> inv(C);
    for (int64_t k = 0; k < C; k++) inv[s->perm[k]] = (int32_t)k;
    std::vector<int32_t> gorder(G);  // device ghost b -> reference ghost
    std::iota(gorder.begin(), gorder.end(), 0);
    std::stable_sort(gorder.begin(), gorder.end(),
                     [&](int32_t a, int32_t b) { return inv[t.e_cell0[t.g_edge[a]]] < inv[t.e_cell0[t.g_edge[b]]]; });
    std::vector<int32_t> gpos(G);
    for (int64_t b = 0; b < G; b++) gpos[gorder[b]] = (int32_t)b;
    std::vector<int32_t> ghost_of_edge(t.E, -1);
    for (int64_t g = 0; g < G; g++) ghost_of_edge[t.g_edge[g]] = (int32_t)g;
    std::vector<int32_t> iedges;
    for (int64_t e2 = 0; e2 < t.E; e2++)
        if (!t.e_boundary[e2]) iedges.push_back((int32_t)e2);
    auto ekey = [&](int32_t e2) {
        int32_t a = inv[t.e_cell0[e2]], b = inv[t.e_cell1[e2]];
        return std::make_pair(std::min(a, b), std::max(a, b));
    };
    std::stable_sort(iedges.begin(), iedges.end(), [&](int32_t a, int32_t b) { return ekey(a) < ekey(b); });
    const int64_t Eint = (int64_t)iedges.size();
    s->Eint = Eint;
    std::vector<int64_t> edev(t.E);  // reference edge -> device flux index
    for (int64_t k = 0; k < Eint; k++) edev[iedges[k]] = k;
    for (int64_t g = 0; g < G; g++) edev[t.g_edge[g]] = Eint + gpos[g];
    auto dev_cell = [&](int32_t c) -> int32_t { return c < C ? inv[c] : (int32_t)(C + gpos[c - C]); };
    auto cen = [&](int32_t c, double &x, double &y) {
        if (c < C) {
            x = t.cx[c];
            y = t.cy[c];
        } else {
            x = t.g_cx[c - C];
            y = t.g_cy[c - C];
        }
    };

    // ---- host images of the device arrays ------------------------------------
    std::vector<int32_t> h_nedge(C), h_snbr(MJ * Cs, 0), h_sedge(MJ * Cs, 0);
    std::vector<double> h_sgm(2 * MJ * Cs, 0), h_snd(2 * MJ * Cs, 0), h_sfd(2 * MJ * Cs, 0);
    std::vector<double> h_nia(C), h_perim(C), h_d(C), h_src;
    std::vector<int32_t> h_eslot(2 * Eint), h_ecell(2 * Eint), h_eref(Eint);
    std::vector<double> h_en(2 * Eint), h_elen(Eint);
    std::vector<int32_t> h_bcell(G), h_bslot(G), h_btype(G), h_bref(G);
    std::vector<double> h_bn(2 * G), h_blen(G), h_brefl(4 * G, 0), h_bdata(4 * G, 0), h_bdq(4 * G, 0), h_bdmid(4 * G, 0);
    std::vector<double> h_grad(8 * (C + G), 0.0);
    std::vector<int32_t> h_cellref(C);
    std::vector<double> h_q(4 * (C + G), 0.0);
    s->ref_nedge.assign(t.nedge.begin(), t.nedge.end());
    std::vector<int64_t> slot_start(C + 1, 0);
    for (int64_t r = 0; r < C; r++) slot_start[r + 1] = slot_start[r] + t.nedge[r];
    s->ref_face_slot.assign(slot_start[C], 0);
    const int mms_kind = cfg->mms ? cfg->mms : EBB_MMS_REFERENCE;
    if (cfg->mms) h_src.assign(4 * C, 0.0);

    for (int64_t i = 0; i < C; i++) {
        const int32_t r = s->perm[i];
        h_cellref[i] = r;
        const int ne = t.nedge[r];
        h_nedge[i] = ne;
        h_nia[i] = -(1.0 / t.area[r]);
        h_perim[i] = t.perim[r];
        h_d[i] = t.d[r];
        for (int j = 0; j < ne; j++) {
            const int64_t sl = (int64_t)r * K + j;
            const int64_t ds = (int64_t)j * Cs + i;
            s->ref_face_slot[slot_start[r] + j] = ds;
            const int32_t nb = t.slot_nbr[sl];
            const int32_t e2 = t.slot_edge[sl];
            h_snbr[ds] = dev_cell(nb);
            int64_t fi = edev[e2];
            h_sedge[ds] = (int32_t)fi | (t.slot_sign[sl] < 0 ? (int32_t)0x80000000 : 0);
            h_sgm[2 * ds] = t.gm0[sl];
            h_sgm[2 * ds + 1] = t.gm1[sl];
            double nx, ny;
            cen(nb, nx, ny);
            h_snd[2 * ds] = nx - t.cx[r];
            h_snd[2 * ds + 1] = ny - t.cy[r];
            h_sfd[2 * ds] = t.e_mx[e2] - t.cx[r];
            h_sfd[2 * ds + 1] = t.e_my[e2] - t.cy[r];
            if (!t.e_boundary[e2]) {
                const int64_t k = fi;
                const int side = (t.e_cell0[e2] == r) ? 0 : 1;
                h_eslot[2 * k + side] = (int32_t)ds;
            } else {
                h_bslot[fi - Eint] = (int32_t)ds;
            }
        }
        if (cfg->mms) {
            double S[4];
            mms_source(cfg->mms, t.cx[r], t.cy[r], *cfg, s->mu, S);
            for (int k = 0; k < 4; k++) h_src[4 * i + k] = S[k];
        }
        // initial conditions (solve.d:196-207; manufactured runs start from the exact field)
        double q0[4];
        if (cfg->mms)
            mms_solution(cfg->mms, t.cx[r], t.cy[r], q0);
        else
            freestream(cfg->ic[0], cfg->ic[1], cfg->ic[3], q0);
        for (int k = 0; k < 4; k++) h_q[4 * i + k] = q0[k];
        if (cfg->order == 1)
            for (int k = 0; k < 8; k++) h_grad[8 * i + k] = NAN;
    }
    for (int64_t k = 0; k < Eint; k++) {
        const int32_t e2 = iedges[k];
        h_ecell[2 * k] = inv[t.e_cell0[e2]];
        h_ecell[2 * k + 1] = inv[t.e_cell1[e2]];
        h_en[2 * k] = t.e_nx[e2];
        h_en[2 * k + 1] = t.e_ny[e2];
        h_elen[k] = t.e_len[e2];
        h_eref[k] = e2;
    }
    bool any_visc_wall = false;
    for (int64_t b = 0; b < G; b++) {
        const int32_t g = gorder[b];
        const int32_t e2 = t.g_edge[g];
        h_bcell[b] = inv[t.e_cell0[e2]];
        h_bn[2 * b] = t.e_nx[e2];
        h_bn[2 * b + 1] = t.e_ny[e2];
        h_blen[b] = t.e_len[e2];
        h_bref[b] = e2;
        const ebb_boundary &B = cfg->boundaries[group_bc[t.e_group[e2]]];
        int type = B.type;
        if (type == EBB_BC_VISCOUS_WALL) any_visc_wall = true;
        const double x1 = mesh->xy[2 * t.e_node0[e2]], y1 = mesh->xy[2 * t.e_node0[e2] + 1];
        const double x2 = mesh->xy[2 * t.e_node1[e2]], y2 = mesh->xy[2 * t.e_node1[e2] + 1];
        if (x1 != x2) {
            double mm = (y2 - y1) / (x2 - x1);
            double den = 1 + mm * mm;
            h_brefl[4 * b] = (1 - mm * mm) * 1.0 / den;
            h_brefl[4 * b + 1] = 2.0 * mm * 1.0 / den;
            h_brefl[4 * b + 2] = 2.0 * mm * 1.0 / den;
            h_brefl[4 * b + 3] = (mm * mm - 1) * 1.0 / den;
        } else {
            type |= 0x100;
        }
        h_btype[b] = type;
        switch (B.type) {
        case EBB_BC_FULL_STATE: {
            double qq[4];
            freestream(B.data[0], B.data[1], B.data[3], qq);
            for (int k = 0; k < 4; k++) h_bdata[4 * b + k] = qq[k];
            break;
        }
        case EBB_BC_CONST_PRESSURE:
            h_bdata[4 * b] = B.data[0];
            break;
        case EBB_BC_TEMP_PRES_INFLOW: {
            double aoa = B.data[2] * M_PI / 180;
            h_bdata[4 * b] = B.data[0];
            h_bdata[4 * b + 1] = B.data[1];
            h_bdata[4 * b + 2] = std::cos(aoa);
            h_bdata[4 * b + 3] = std::sin(aoa);
            break;
        }
        case EBB_BC_DIRICHLET: {
            double qq[4], gg[4][2];
            mms_solution(mms_kind, t.g_cx[g], t.g_cy[g], qq);
            for (int k = 0; k < 4; k++) h_bdq[4 * b + k] = qq[k];
            mms_solution(mms_kind, t.e_mx[e2], t.e_my[e2], qq);
            for (int k = 0; k < 4; k++) h_bdmid[4 * b + k] = qq[k];
            mms_gradient(mms_kind, t.g_cx[g], t.g_cy[g], gg);
            for (int k = 0; k < 4; k++) {
                h_grad[8 * (C + b) + 2 * k] = gg[k][0];
                h_grad[8 * (C + b) + 2 * k + 1] = gg[k][1];
            }
            break;
        }
        default:
            break;
        }
    }
    // force edges: all boundary edges of the first group named by each force tag (mesh.d:645-671)
    std::vector<int32_t> h_force;
    for (int f = 0; f < cfg->n_force; f++) {
        int g = -1;
        for (int k = 0; k < nG; k++)
            if (mesh->tags[k] == cfg->force_boundary[f]) {
                g = k;
                break;
            }
        if (g < 0) continue;
        for (int64_t gg = 0; gg < G; gg++)
            if (t.e_group[t.g_edge[gg]] == g) h_force.push_back(gpos[gg]);
    }

    // ---- device allocation (one arena) ----------------------------------------
    const bool split = precision == EBB_PREC_SPLIT;
    const size_t rs = split ? sizeof(float) : sizeof(double);  // bytes of the arithmetic type
    const int64_t NQ = C + G;
    s->nred = update_blocks((int)C);
    auto rsz = [&](size_t n) { return ((n * rs) + 255) & ~(size_t)255; };
    size_t total = 0;
    total += sz<double>(4 * NQ);                                        // q64
    total += split ? rsz(4 * NQ) : 0;                                   // qs1 (float shadow)
    total += 2 * rsz(4 * NQ);                                           // qs, aux
    total += rsz(4 * MJ * Cs) + rsz(8 * NQ);                            // face, grad
    total += rsz(4 * (Eint + G)) + rsz(Eint + G) + rsz(C);              // fl, fs, cdt
    total += sz<double>(8 * (size_t)s->nred) + sz<DState>(1) + sz<DRecord>(EBB_REC_CAP);
    total += 3 * sz<int32_t>(C) + 3 * rsz(C) + (cfg->mms ? rsz(4 * C) : 0);
    total += 2 * sz<int32_t>(MJ * Cs) + 3 * rsz(2 * MJ * Cs);
    total += 2 * sz<int32_t>(2 * Eint) + rsz(2 * Eint) + rsz(Eint) + sz<int32_t>(Eint);
    total += 4 * sz<int32_t>(G) + rsz(2 * G) + rsz(G) + 4 * rsz(4 * G);
    total += sz<int32_t>(h_force.size() + 1);
    total += 2 * sz<double>(4 * C);  // host-order staging, device-order scratch
    s->dbytes = total;
    cudaError_t ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaMalloc(&s->dmem, total);
    if (ce != cudaSuccess) {
        set_err(err, err_len, std::string("CUDA: ") + cudaGetErrorString(ce));
        int code = ce == cudaErrorMemoryAllocation ? EBB_ERR_OOM : EBB_ERR_CUDA;
        ebb_solver_destroy(s);
        return code;
    }
    cudaMemsetAsync(s->dmem, 0, total, s->stream);
    Arena ar{(char *)s->dmem, 0, total};
    DArrays &A = s->A;
    auto takeR = [&](size_t n) -> void * { return split ? (void *)ar.take<float>(n) : (void *)ar.take<double>(n); };
    A.q64 = ar.take<double>(4 * NQ);
    A.qs1 = split ? takeR(4 * NQ) : (void *)A.q64;
    A.qs = takeR(4 * NQ);
    A.aux = takeR(4 * NQ);
    A.face = takeR(4 * MJ * Cs);
    A.grad = takeR(8 * NQ);
    A.fl = takeR(4 * (Eint + G));
    A.fs = takeR(Eint + G);
    A.cdt = takeR(C);
    A.red = ar.take<double>(8 * (size_t)s->nred);
    A.st = ar.take<DState>(1);
    A.rec = ar.take<DRecord>(EBB_REC_CAP);
    A.R = A.aux;
    DMesh &M = s->M;
    M.C = (int32_t)C;
    M.G = (int32_t)G;
    M.Cs = (int32_t)Cs;
    M.Eint = (int32_t)Eint;
    M.maxJ = MJ;
    auto up = [&](auto *dst, const auto &v) {
        if (!v.empty()) cudaMemcpyAsync((void *)dst, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice, s->stream);
        return dst;
    };
    // real arrays: FP64 precompute, stored in the arithmetic type
    auto upR = [&](const std::vector<double> &v) -> const void * {
        void *dst = takeR(v.size() ? v.size() : 1);
        if (v.empty()) return dst;
        if (split) {
            std::vector<float> f(v.begin(), v.end());
            cudaMemcpyAsync(dst, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream);
            cudaStreamSynchronize(s->stream);
        } else {
            cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream);
        }
        return dst;
    };
    int32_t *p_nedge = ar.take<int32_t>(C);
    M.nedge = up(p_nedge, h_nedge);
    int32_t *p_cellref = ar.take<int32_t>(C);
    M.cell_ref = up(p_cellref, h_cellref);
    s->d_perm = ar.take<int32_t>(C);
    up(s->d_perm, h_cellref);
    M.g.neg_inv_area = upR(h_nia);
    M.g.perim = upR(h_perim);
    M.g.dlen = upR(h_d);
    M.g.src = cfg->mms ? upR(h_src) : nullptr;
    int32_t *pi;
    pi = ar.take<int32_t>(MJ * Cs);
    M.s_nbr = up(pi, h_snbr);
    pi = ar.take<int32_t>(MJ * Cs);
    M.s_edge = up(pi, h_sedge);
    M.g.s_gm = upR(h_sgm);
    M.g.s_nd = upR(h_snd);
    M.g.s_fd = upR(h_sfd);
    pi = ar.take<int32_t>(2 * Eint);
    M.e_slot = up(pi, h_eslot);
    pi = ar.take<int32_t>(2 * Eint);
    M.e_cell = up(pi, h_ecell);
    M.g.e_n = upR(h_en);
    M.g.e_len = upR(h_elen);
    pi = ar.take<int32_t>(Eint);
    M.e_ref = up(pi, h_eref);
    pi = ar.take<int32_t>(G);
    M.b_cell = up(pi, h_bcell);
    pi = ar.take<int32_t>(G);
    M.b_slot = up(pi, h_bslot);
    pi = ar.take<int32_t>(G);
    M.b_type = up(pi, h_btype);
    pi = ar.take<int32_t>(G);
    M.b_ref = up(pi, h_bref);
    M.g.b_n = upR(h_bn);
    M.g.b_len = upR(h_blen);
    M.g.b_refl = upR(h_brefl);
    M.g.b_data = upR(h_bdata);
    M.g.b_dq = upR(h_bdq);
    M.g.b_dmid = upR(h_bdmid);
    pi = ar.take<int32_t>(h_force.size() + 1);
    M.force_b = up(pi, h_force);
    M.n_force = (int32_t)h_force.size();
    s->d_stage = ar.take<double>(4 * C);
    s->d_tmp = ar.take<double>(4 * C);
    up(A.q64, h_q);
    if (split) {
        std::vector<float> gf(h_grad.begin(), h_grad.end());
        cudaMemcpyAsync(A.grad, gf.data(), gf.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream);
        cudaStreamSynchronize(s->stream);
        launch_to_float4(A.q64, reinterpret_cast<float *>(A.qs1), C, s->stream);
    } else {
        up(reinterpret_cast<double *>(A.grad), h_grad);
    }

    DPhys &P = s->P;
    P.flux = cfg->flux;
    P.limited = cfg->limited;
    P.order = (int32_t)cfg->order;
    P.viscous = cfg->viscosity;
    P.mms = cfg->mms;
    P.local_ts = cfg->local_timestep;
    P.lp = (cfg->lp_thresh > 0) ? 1 : 0;
    P.lp_thresh = cfg->lp_thresh;
    P.pr = cfg->pr;
    P.mu = s->mu;
    P.r_gas = cfg->r_gas;
    P.need_grad = (cfg->viscosity || any_visc_wall) ? 1 : 0;

    DState h{};
    h.dt = cfg->dt;
    h.t = 0;
    h.cfl = cfg->cfl;
    h.t_end = cfg->t_end;
    h.dt_half = h.dt / 2.0;
    h.dt_sixth = h.dt / 6.0;
    h.dtf = (float)h.dt;
    h.dt_half_f = (float)h.dt_half;
    h.dt_sixth_f = (float)h.dt_sixth;
    h.newdt_bits = 0x7FF0000000000000ull;
    h.rmax_bits = 0;
    h.err_key = EBB_NOERR;
    h.resid_last = INFINITY;
    h.resid_inc = 0;
    h.done = !(h.t < h.t_end);
    h.iter = 0;
    h.dynamic_dt = cfg->dynamic_dt;
    h.cfl_adjust = cfg->cfl_adjust;
    double aoa = cfg->ic[1] * (M_PI / 180);
    h.rot[0] = std::cos(aoa);
    h.rot[1] = -std::sin(aoa);
    h.rot[2] = std::sin(aoa);
    h.rot[3] = std::cos(aoa);
    h.n_rec = 0;
    h.rec_enabled = 1;
    cudaMemcpyAsync(A.st, &h, sizeof h, cudaMemcpyHostToDevice, s->stream);
    ce = cudaStreamSynchronize(s->stream);
    if (ce != cudaSuccess) {
        set_err(err, err_len, std::string("CUDA: ") + cudaGetErrorString(ce));
        ebb_solver_destroy(s);
        return EBB_ERR_CUDA;
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
    CK(cudaMemcpyAsync(s->d_stage, q, sizeof(double) * 4 * s->C, cudaMemcpyHostToDevice, s->stream));
    CKL(launch_permute4(s->d_stage, s->A.q64, s->d_perm, s->C, 1, s->stream));
    if (s->precision == EBB_PREC_SPLIT)
        CKL(launch_to_float4(s->A.q64, reinterpret_cast<float *>(s->A.qs1), s->C, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
}

int ebb_get_state(ebb_solver *s, double *q)
{
    if (!s || !q) return EBB_ERR_ARG;
    CKL(launch_permute4(s->A.q64, s->d_stage, s->d_perm, s->C, 0, s->stream));
    CK(cudaMemcpyAsync(q, s->d_stage, sizeof(double) * 4 * s->C, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return EBB_OK;
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
    h.dt = dt;
    h.dt_half = dt / 2.0;
    h.dt_sixth = dt / 6.0;
    h.dtf = (float)dt;
    h.dt_half_f = (float)h.dt_half;
    h.dt_sixth_f = (float)h.dt_sixth;
    h.done = !(h.t < h.t_end);
    return solver_write_state(s, h);
}

int ebb_residual(ebb_solver *s, const double *q, double *R, double *new_dt, double *rmax, int32_t limit,
                 int32_t dt_update)
{
    if (!s || !q || !R) return EBB_ERR_ARG;
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
    const bool split = s->precision == EBB_PREC_SPLIT;
    if (split) {
        CKL(launch_permute4(q_dev, s->d_tmp, s->d_perm, s->C, 1, s->stream));
        CKL(launch_to_float4(s->d_tmp, reinterpret_cast<float *>(s->A.qs), s->C, s->stream));
    } else {
        CKL(launch_permute4(q_dev, reinterpret_cast<double *>(s->A.qs), s->d_perm, s->C, 1, s->stream));
    }
    int r = solver_run_residual_on_qs(s, limit, dt_update, new_dt, rmax);
    if (r) return r;
    if (split) {
        CKL(launch_to_double4(reinterpret_cast<const float *>(s->A.R), s->d_tmp, s->C, s->stream));
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
    DState h;
    int r = solver_sync_state(s, h);
    if (r) return r;
    const int saved_done = h.done;
    h.dt = *dt;
    h.dt_half = *dt / 2.0;
    h.dt_sixth = *dt / 6.0;
    h.dtf = (float)*dt;
    h.dt_half_f = (float)h.dt_half;
    h.dt_sixth_f = (float)h.dt_sixth;
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
    DState h;
    int r = solver_sync_state(s, h);
    if (r) return r;
    if (h.err_key != EBB_NOERR) return decode_error(s, h);
    if (h.done) return EBB_OK;
    if (!s->g1 && (r = build_graph(s, 1, &s->g1))) return r;
    if (!s->g16 && (r = build_graph(s, 16, &s->g16))) return r;
    int64_t run = 0;
    while (run < max_steps) {
        const int64_t chunk = std::min<int64_t>(max_steps - run, EBB_REC_CAP);
        const int64_t it0 = h.iter, rec0 = h.n_rec;
        int64_t k = 0;
        for (; k + 16 <= chunk; k += 16) CK(cudaGraphLaunch(s->g16, s->stream));
        for (; k < chunk; k++) CK(cudaGraphLaunch(s->g1, s->stream));
        if ((r = solver_sync_state(s, h))) return r;
        const int64_t did = h.iter - it0;
        if (records && h.n_rec > rec0) {
            for (int64_t m = rec0; m < h.n_rec; m++) {
                CK(cudaMemcpyAsync(&records[run + (m - rec0)], &s->A.rec[m % EBB_REC_CAP], sizeof(DRecord),
                                   cudaMemcpyDeviceToHost, s->stream));
            }
            CK(cudaStreamSynchronize(s->stream));
        }
        run += did;
        if (h.err_key != EBB_NOERR) {
            if (steps_run) *steps_run = run;
            return decode_error(s, h);
        }
        if (h.done || did < chunk) break;
    }
    if (steps_run) *steps_run = run;
    return EBB_OK;
}

int ebb_run_timed(ebb_solver *s, int64_t max_steps, int64_t *steps_run, double *device_ms)
{
    if (!s || max_steps < 0 || !device_ms) return EBB_ERR_ARG;
    if (steps_run) *steps_run = 0;
    *device_ms = 0;
    DState h;
    int r = solver_sync_state(s, h);
    if (r) return r;
    if (h.err_key != EBB_NOERR) return decode_error(s, h);
    if (!s->g1 && (r = build_graph(s, 1, &s->g1))) return r;
    if (!s->g16 && (r = build_graph(s, 16, &s->g16))) return r;
    const int64_t it0 = h.iter;
    cudaEvent_t ev[2];
    CK(cudaEventCreate(&ev[0]));
    CK(cudaEventCreate(&ev[1]));
    CK(cudaEventRecord(ev[0], s->stream));
    int64_t k = 0;
    for (; k + 16 <= max_steps; k += 16) CK(cudaGraphLaunch(s->g16, s->stream));
    for (; k < max_steps; k++) CK(cudaGraphLaunch(s->g1, s->stream));
    CK(cudaEventRecord(ev[1], s->stream));
    CK(cudaEventSynchronize(ev[1]));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    *device_ms = ms;
    if ((r = solver_sync_state(s, h))) return r;
    if (steps_run) *steps_run = h.iter - it0;
    return decode_error(s, h);
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
    DState h0;
    int r = solver_sync_state(s, h0);
    if (r) return r;
    DState h = h0;
    h.done = 0;
    h.err_key = EBB_NOERR;
    h.rec_enabled = 0;
    if ((r = solver_write_state(s, h))) return r;
    r = s->precision == EBB_PREC_SPLIT ? profile_t<float>(s, n_rep, ms) : profile_t<double>(s, n_rep, ms);
    int r2 = solver_write_state(s, h0);
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
    } else {
        CK(cudaMemcpyAsync(f.data(), s->A.face, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    for (size_t k = 0; k < s->ref_face_slot.size(); k++)
        for (int c = 0; c < 4; c++) out[4 * k + c] = f[4 * s->ref_face_slot[k] + c];
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
    cudaMemcpy(dL, qL, sizeof(double) * 4 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dR, qR, sizeof(double) * 4 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dn, normal, sizeof(double) * 2 * n, cudaMemcpyHostToDevice);
    int r = launch_flux_batch(kind, n, dL, dR, dn, dF, ds, nullptr);
    cudaError_t e = cudaMemcpy(F, dF, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(s_max, ds, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (r || e != cudaSuccess) return EBB_ERR_CUDA;
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
