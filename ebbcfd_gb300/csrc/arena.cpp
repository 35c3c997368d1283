// arena.cpp -- device layout of one or many meshes (buildMesh + ufvmSetup per instance,
// source/mesh.d:217-643 and source/solve.d:175-279), assembled into one arena.
//
// Each instance is laid out on its own first (Hilbert cell order, ghosts by owner, interior
// edges by first cell, FP64 geometry), in local numbering.  The arena concatenates the
// instances: interior cells of every instance first, then every instance's ghost
// cells, interior edges first then boundary edges, face slots in one ELL array whose
// stride is the total cell count.  The kernels see one mesh; instance boundaries only
// matter to the per-instance time-loop state (dt, t, CFL, reductions, stop condition),
// which the update kernel reaches through a block -> instance table (blocks never
// straddle two instances) and the step-end kernel through one block per instance.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "solver_impl.hpp"
#include "tuned.h"

namespace ebb {
namespace {

constexpr int K = kMaxEdges;
constexpr int UPD = EBB_UPD_TB;  // k_update threads per block (the tuned value the kernels use)

template <typename T> size_t sz(size_t n) { return ((n * sizeof(T)) + 255) & ~(size_t)255; }

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

}  // namespace

int build_instance(const ebb_mesh *mesh, const ebb_config *cfg, InstLayout &L, std::string &e)
{
    Topology t;
    if (!build_topology(*mesh, t, e)) return EBB_ERR_MESH;
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
            e = "Could not find matching boundary condition tag " + mesh->tags[g];
            return EBB_ERR_CONFIG;
        }
        const ebb_boundary &B = cfg->boundaries[group_bc[g]];
        if (B.type == EBB_BC_CONST_PRESSURE && B.n_data != 1) {
            e = "Constant pressure boundary data should only have one element; the constant pressure";
            return EBB_ERR_CONFIG;
        }
        if (B.type == EBB_BC_TEMP_PRES_INFLOW && B.n_data != 3) {
            e = "Constant temperature/pressure/aoa boundary data should have three elements";
            return EBB_ERR_CONFIG;
        }
        if (B.type == EBB_BC_FULL_STATE && B.n_data < 4) {
            e = "fullState boundary data needs [M, aoa, p, rho]";
            return EBB_ERR_CONFIG;
        }
    }
    L.cfg = *cfg;
    const int64_t C = t.C, G = t.G;
    L.C = C;
    L.G = G;
    L.maxJ = t.maxJ;
    L.mu = cfg->viscosity ? (cfg->ic[3] * 1.0 * cfg->l_ref) / cfg->re : NAN;

    // ---- orderings ----------------------------------------------------------
    L.perm = hilbert_order(t);
    std::vector<int32_t> inv(C);
    for (int64_t k = 0; k < C; k++) inv[L.perm[k]] = (int32_t)k;
    std::vector<int32_t> gorder(G);  // local ghost b -> reference ghost
    std::iota(gorder.begin(), gorder.end(), 0);
    std::stable_sort(gorder.begin(), gorder.end(),
                     [&](int32_t a, int32_t b) { return inv[t.e_cell0[t.g_edge[a]]] < inv[t.e_cell0[t.g_edge[b]]]; });
    std::vector<int32_t> gpos(G);
    for (int64_t b = 0; b < G; b++) gpos[gorder[b]] = (int32_t)b;
    std::vector<int32_t> iedges;
    for (int64_t e2 = 0; e2 < t.E; e2++)
        if (!t.e_boundary[e2]) iedges.push_back((int32_t)e2);
    auto ekey = [&](int32_t e2) {
        int32_t a = inv[t.e_cell0[e2]], b = inv[t.e_cell1[e2]];
        return std::make_pair(std::min(a, b), std::max(a, b));
    };
    std::stable_sort(iedges.begin(), iedges.end(), [&](int32_t a, int32_t b) { return ekey(a) < ekey(b); });
    const int64_t Eint = (int64_t)iedges.size();
    L.Eint = Eint;
    std::vector<int64_t> edev(t.E);  // reference edge -> local flux index
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

    // ---- local images (slot (i, j) at j*C + i) ------------------------------------
    const int MJ = t.maxJ;
    L.nedge.resize(C);
    L.cellref.resize(C);
    L.nia.resize(C);
    L.perim.resize(C);
    L.d.resize(C);
    L.snbr.assign(MJ * C, 0);
    L.sedge.assign(MJ * C, 0);
    L.sgm.assign(2 * MJ * C, 0);
    L.snd.assign(2 * MJ * C, 0);
    L.sfd.assign(2 * MJ * C, 0);
    L.eslot.resize(2 * Eint);
    L.ecell.resize(2 * Eint);
    L.eref.resize(Eint);
    L.en.resize(2 * Eint);
    L.elen.resize(Eint);
    L.bcell.resize(G);
    L.bslot.resize(G);
    L.btype.resize(G);
    L.bref.resize(G);
    L.bn.resize(2 * G);
    L.blen.resize(G);
    L.brefl.assign(4 * G, 0);
    L.bdata.assign(4 * G, 0);
    L.bdq.assign(4 * G, 0);
    L.bdmid.assign(4 * G, 0);
    L.grad.assign(8 * (C + G), 0.0);
    L.q.assign(4 * C, 0.0);
    L.ref_nedge.assign(t.nedge.begin(), t.nedge.end());
    std::vector<int64_t> slot_start(C + 1, 0);
    for (int64_t r = 0; r < C; r++) slot_start[r + 1] = slot_start[r] + t.nedge[r];
    L.ref_face_slot.assign(slot_start[C], 0);
    const int mms_kind = cfg->mms ? cfg->mms : EBB_MMS_REFERENCE;
    if (cfg->mms) L.src.assign(4 * C, 0.0);

    for (int64_t i = 0; i < C; i++) {
        const int32_t r = L.perm[i];
        L.cellref[i] = r;
        const int ne = t.nedge[r];
        L.nedge[i] = ne;
        L.nia[i] = -(1.0 / t.area[r]);
        L.perim[i] = t.perim[r];
        L.d[i] = t.d[r];
        for (int j = 0; j < ne; j++) {
            const int64_t sl = (int64_t)r * K + j;
            const int64_t ds = (int64_t)j * C + i;
            L.ref_face_slot[slot_start[r] + j] = ds;
            const int32_t nb = t.slot_nbr[sl];
            const int32_t e2 = t.slot_edge[sl];
            L.snbr[ds] = dev_cell(nb);
            const int64_t fi = edev[e2];
            L.sedge[ds] = (int32_t)fi | (t.slot_sign[sl] < 0 ? (int32_t)0x80000000 : 0);
            L.sgm[2 * ds] = t.gm0[sl];
            L.sgm[2 * ds + 1] = t.gm1[sl];
            double nx, ny;
            cen(nb, nx, ny);
            L.snd[2 * ds] = nx - t.cx[r];
            L.snd[2 * ds + 1] = ny - t.cy[r];
            L.sfd[2 * ds] = t.e_mx[e2] - t.cx[r];
            L.sfd[2 * ds + 1] = t.e_my[e2] - t.cy[r];
            if (!t.e_boundary[e2])
                L.eslot[2 * fi + ((t.e_cell0[e2] == r) ? 0 : 1)] = (int32_t)ds;
            else
                L.bslot[fi - Eint] = (int32_t)ds;
        }
        if (cfg->mms) {
            double S[4];
            mms_source(cfg->mms, t.cx[r], t.cy[r], *cfg, L.mu, S);
            for (int k = 0; k < 4; k++) L.src[4 * i + k] = S[k];
        }
        // initial conditions (solve.d:196-207; manufactured runs start from the exact field)
        double q0[4];
        if (cfg->mms)
            mms_solution(cfg->mms, t.cx[r], t.cy[r], q0);
        else
            freestream(cfg->ic[0], cfg->ic[1], cfg->ic[3], q0);
        for (int k = 0; k < 4; k++) L.q[4 * i + k] = q0[k];
        if (cfg->order == 1)
            for (int k = 0; k < 8; k++) L.grad[8 * i + k] = NAN;
    }
    for (int64_t k = 0; k < Eint; k++) {
        const int32_t e2 = iedges[k];
        L.ecell[2 * k] = inv[t.e_cell0[e2]];
        L.ecell[2 * k + 1] = inv[t.e_cell1[e2]];
        L.en[2 * k] = t.e_nx[e2];
        L.en[2 * k + 1] = t.e_ny[e2];
        L.elen[k] = t.e_len[e2];
        L.eref[k] = e2;
    }
    L.any_visc_wall = false;
    for (int64_t b = 0; b < G; b++) {
        const int32_t g = gorder[b];
        const int32_t e2 = t.g_edge[g];
        L.bcell[b] = inv[t.e_cell0[e2]];
        L.bn[2 * b] = t.e_nx[e2];
        L.bn[2 * b + 1] = t.e_ny[e2];
        L.blen[b] = t.e_len[e2];
        L.bref[b] = e2;
        const ebb_boundary &B = cfg->boundaries[group_bc[t.e_group[e2]]];
        int type = B.type;
        if (type == EBB_BC_VISCOUS_WALL) L.any_visc_wall = true;
        const double x1 = mesh->xy[2 * t.e_node0[e2]], y1 = mesh->xy[2 * t.e_node0[e2] + 1];
        const double x2 = mesh->xy[2 * t.e_node1[e2]], y2 = mesh->xy[2 * t.e_node1[e2] + 1];
        if (x1 != x2) {
            double mm = (y2 - y1) / (x2 - x1);
            double den = 1 + mm * mm;
            L.brefl[4 * b] = (1 - mm * mm) * 1.0 / den;
            L.brefl[4 * b + 1] = 2.0 * mm * 1.0 / den;
            L.brefl[4 * b + 2] = 2.0 * mm * 1.0 / den;
            L.brefl[4 * b + 3] = (mm * mm - 1) * 1.0 / den;
        } else {
            type |= 0x100;
        }
        L.btype[b] = type;
        switch (B.type) {
        case EBB_BC_FULL_STATE: {
            double qq[4];
            freestream(B.data[0], B.data[1], B.data[3], qq);
            for (int k = 0; k < 4; k++) L.bdata[4 * b + k] = qq[k];
            break;
        }
        case EBB_BC_CONST_PRESSURE:
            L.bdata[4 * b] = B.data[0];
            break;
        case EBB_BC_TEMP_PRES_INFLOW: {
            double aoa = B.data[2] * M_PI / 180;
            L.bdata[4 * b] = B.data[0];
            L.bdata[4 * b + 1] = B.data[1];
            L.bdata[4 * b + 2] = std::cos(aoa);
            L.bdata[4 * b + 3] = std::sin(aoa);
            break;
        }
        case EBB_BC_DIRICHLET: {
            double qq[4], gg[4][2];
            mms_solution(mms_kind, t.g_cx[g], t.g_cy[g], qq);
            for (int k = 0; k < 4; k++) L.bdq[4 * b + k] = qq[k];
            mms_solution(mms_kind, t.e_mx[e2], t.e_my[e2], qq);
            for (int k = 0; k < 4; k++) L.bdmid[4 * b + k] = qq[k];
            mms_gradient(mms_kind, t.g_cx[g], t.g_cy[g], gg);
            for (int k = 0; k < 4; k++) {
                L.grad[8 * (C + b) + 2 * k] = gg[k][0];
                L.grad[8 * (C + b) + 2 * k + 1] = gg[k][1];
            }
            break;
        }
        default:
            break;
        }
    }
    // force edges: all boundary edges of the first group named by each force tag (mesh.d:645-671)
    for (int f = 0; f < cfg->n_force; f++) {
        int g = -1;
        for (int k = 0; k < nG; k++)
            if (mesh->tags[k] == cfg->force_boundary[f]) {
                g = k;
                break;
            }
        if (g < 0) continue;
        for (int64_t gg = 0; gg < G; gg++)
            if (t.e_group[t.g_edge[gg]] == g) L.force.push_back(gpos[gg]);
    }

    // time-loop state (app/solver.d:43-50)
    DState &h = L.st0;
    std::memset(&h, 0, sizeof h);
    set_step(h, cfg->dt);
    h.t = 0;
    h.cfl = cfg->cfl;
    h.cflf = (float)h.cfl;
    h.t_end = cfg->t_end;
    h.newdt_bits = 0x7FF0000000000000ull;
    h.rmax_bits = 0;
    h.err_key = EBB_NOERR;
    h.resid_last = INFINITY;
    h.stall_steps = 0;
    h.resid_min = INFINITY;
    h.resid_min_iter = 0;
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
    h.max_steps = 0;
    h.stop_drop = 0;
    h.resid_first = -1;
    return EBB_OK;
}

// Physics shared by every instance of an arena: one DPhys per launch.
static bool same_physics(const ebb_config &a, const ebb_config &b)
{
    return a.flux == b.flux && a.integrator == b.integrator && a.limited == b.limited && a.order == b.order &&
           a.viscosity == b.viscosity && a.local_timestep == b.local_timestep &&
           a.multistage_limiting == b.multistage_limiting && (a.lp_thresh > 0) == (b.lp_thresh > 0) &&
           (!(a.lp_thresh > 0) || a.lp_thresh == b.lp_thresh) && a.mms == b.mms && a.pr == b.pr &&
           a.r_gas == b.r_gas;
}

namespace {

struct Dims {
    int n = 0;
    int64_t Ct = 0, Gt = 0, Et = 0, Cs = 0, nforce = 0;
    int MJ = 0, nblk = 0;
    bool any_mms = false, visc_wall = false;
};

Dims dims_of(const std::vector<InstLayout> &Ls)
{
    Dims D;
    D.n = (int)Ls.size();
    for (const InstLayout &L : Ls) {
        D.Ct += L.C;
        D.Gt += L.G;
        D.Et += L.Eint;
        D.nforce += (int64_t)L.force.size();
        D.MJ = std::max(D.MJ, L.maxJ);
        D.visc_wall |= L.any_visc_wall;
        D.any_mms |= L.cfg.mms != 0;
        D.nblk += (int)((L.C + UPD - 1) / UPD);
    }
    // slot rows up to the kernels' compiled neighbour count (3, 4 or 6): the stage
    // kernels load every row unconditionally and select by the cell's edge count
    D.MJ = D.MJ <= 3 ? 3 : (D.MJ == 4 ? 4 : 6);
    D.Cs = (D.Ct + 31) & ~(int64_t)31;
    if (D.n == 1) D.nblk = update_blocks((int)D.Ct);
    return D;
}

// device bytes of one arena (every array rounded up to 256 bytes)
size_t bytes_of(const Dims &D, int32_t precision)
{
    const bool split = precision == EBB_PREC_SPLIT;
    const bool dfp = precision == EBB_PREC_DF;
    const size_t rs = split ? sizeof(float) : sizeof(double);  // a double-float is 8 bytes too
    auto rsz = [&](size_t m) { return ((m * rs) + 255) & ~(size_t)255; };
    const int64_t NQ = D.Ct + D.Gt, MJ = D.MJ, Cs = D.Cs, Ct = D.Ct, Gt = D.Gt, Et = D.Et;
    const int n = D.n;
    size_t total = 0;
    total += sz<double>(4 * NQ);                           // q64
    total += (split || dfp) ? rsz(4 * NQ) : 0;             // qs1 (FP32 or double-float shadow)
    total += 2 * rsz(4 * NQ);                              // qs, aux
    total += rsz(4 * MJ * Cs) + rsz(8 * NQ);               // face, grad
    total += rsz(4 * (Et + Gt)) + rsz(Et + Gt) + rsz(Ct);  // fl, fs, cdt
    total += sz<double>(8 * (size_t)D.nblk) + sz<DState>(n) + sz<DRecord>(EBB_REC_CAP);
    total += 4 * sz<int32_t>(Ct) + 3 * rsz(Ct) + (D.any_mms ? rsz(4 * Ct) : 0);
    total += 2 * sz<int32_t>(MJ * Cs) + 3 * rsz(2 * MJ * Cs);
    total += split ? rsz(2 * MJ * Cs) + rsz(MJ * Cs) : 0;  // per-slot edge normal and length
    total += 2 * sz<int32_t>(2 * Et) + rsz(2 * Et) + rsz(Et) + sz<int32_t>(Et);
    total += 4 * sz<int32_t>(Gt) + rsz(2 * Gt) + rsz(Gt) + 4 * rsz(4 * Gt);
    total += sz<int32_t>(D.nforce + 1) + sz<int32_t>(n + 1);
    total += 2 * sz<double>(4 * Ct);  // host-order staging, device-order scratch
    if (n > 1) total += sz<int32_t>(Ct) + 3 * sz<int32_t>(D.nblk) + 2 * sz<int32_t>(n + 1) + sz<double>(n) + sz<float>(n);
    return total + 32 * 256;  // empty arrays still take one 256-byte unit each
}

}  // namespace

size_t arena_bytes(const std::vector<InstLayout> &Ls, int32_t precision) { return bytes_of(dims_of(Ls), precision); }

int assemble(ebb_solver *s, std::vector<InstLayout> &Ls, int32_t precision, std::string &e)
{
    const int n = (int)Ls.size();
    for (int k = 1; k < n; k++)
        if (!same_physics(Ls[0].cfg, Ls[k].cfg)) {
            e = "instances of one arena must share flux, integrator, limiter, order, viscosity and MMS settings";
            return EBB_ERR_CONFIG;
        }
    const Dims D = dims_of(Ls);
    if (D.Ct > INT32_MAX / 8 || (int64_t)D.MJ * D.Cs > INT32_MAX / 2 || D.Et + D.Gt > INT32_MAX / 8) {
        e = "arena too large for 32-bit indices";
        return EBB_ERR_LIMIT;
    }
    s->cfg = Ls[0].cfg;
    s->precision = precision;
    s->n_inst = n;
    s->inst.resize(n);
    {
        int64_t c = 0, g = 0, ed = 0;
        for (int k = 0; k < n; k++) {
            InstMeta &m = s->inst[k];
            m.c0 = c;
            m.C = Ls[k].C;
            m.g0 = g;
            m.G = Ls[k].G;
            m.e0 = ed;
            m.Eint = Ls[k].Eint;
            m.cfg = Ls[k].cfg;
            c += Ls[k].C;
            g += Ls[k].G;
            ed += Ls[k].Eint;
        }
    }
    const int64_t Ct = D.Ct, Gt = D.Gt, Et = D.Et, Cs = D.Cs;
    const int MJ = D.MJ;
    const bool any_mms = D.any_mms, visc_wall = D.visc_wall;
    s->C = Ct;
    s->G = Gt;
    s->Eint = Et;
    s->Cs = Cs;
    s->maxJ = MJ;
    s->mu = Ls[0].mu;

    // ---- global host images ----------------------------------------------------
    std::vector<int32_t> nedge(Ct), cellref(Ct), snbr(MJ * Cs, 0), sedge(MJ * Cs, 0);
    std::vector<double> nia(Ct), perim(Ct), d(Ct), src(any_mms ? 4 * Ct : 0);
    std::vector<double> sgm(2 * MJ * Cs, 0), snd(2 * MJ * Cs, 0), sfd(2 * MJ * Cs, 0);
    std::vector<int32_t> eslot(2 * Et), ecell(2 * Et), eref(Et);
    std::vector<double> en(2 * Et), elen(Et);
    std::vector<int32_t> bcell(Gt), bslot(Gt), btype(Gt), bref(Gt);
    std::vector<double> bn(2 * Gt), blen(Gt), brefl(4 * Gt), bdata(4 * Gt), bdq(4 * Gt), bdmid(4 * Gt);
    std::vector<double> grad(8 * (Ct + Gt)), q(4 * (Ct + Gt), 0.0);
    std::vector<int32_t> force, force_off(n + 1, 0), cell_inst(n > 1 ? Ct : 0);
    std::vector<int32_t> blk_first, blk_end, blk_inst, inst_blk(n + 1, 0), inst_c0(n + 1, 0);
    std::vector<double> inst_mu(n);
    std::vector<float> inst_muf(n);
    s->perm.resize(Ct);
    s->ref_face_slot.clear();
    s->ref_nedge.clear();
    for (int k = 0; k < n; k++) {
        const InstLayout &L = Ls[k];
        const InstMeta &m = s->inst[k];
        const int64_t C = L.C, c0 = m.c0, g0 = m.g0, e0 = m.e0;
        auto gcell = [&](int32_t x) -> int32_t { return x < C ? (int32_t)(c0 + x) : (int32_t)(Ct + g0 + (x - C)); };
        auto gslot = [&](int64_t sl) -> int32_t { return (int32_t)((sl / C) * Cs + c0 + (sl % C)); };
        auto gflux = [&](int32_t f) -> int32_t {
            const int32_t sign = f & (int32_t)0x80000000;
            const int32_t x = f & 0x7fffffff;
            return (x < L.Eint ? (int32_t)(e0 + x) : (int32_t)(Et + g0 + (x - L.Eint))) | sign;
        };
        for (int64_t i = 0; i < C; i++) {
            nedge[c0 + i] = L.nedge[i];
            cellref[c0 + i] = L.cellref[i];  // error reports name the cell within its instance
            s->perm[c0 + i] = (int32_t)(c0 + L.perm[i]);
            nia[c0 + i] = L.nia[i];
            perim[c0 + i] = L.perim[i];
            d[c0 + i] = L.d[i];
            if (L.cfg.mms)
                for (int c = 0; c < 4; c++) src[4 * (c0 + i) + c] = L.src[4 * i + c];
            for (int c = 0; c < 4; c++) q[4 * (c0 + i) + c] = L.q[4 * i + c];
            for (int c = 0; c < 8; c++) grad[8 * (c0 + i) + c] = L.grad[8 * i + c];
            if (n > 1) cell_inst[c0 + i] = k;
            for (int j = 0; j < L.nedge[i]; j++) {
                const int64_t ls = (int64_t)j * C + i, gs = (int64_t)j * Cs + c0 + i;
                snbr[gs] = gcell(L.snbr[ls]);
                sedge[gs] = gflux(L.sedge[ls]);
                for (int c = 0; c < 2; c++) {
                    sgm[2 * gs + c] = L.sgm[2 * ls + c];
                    snd[2 * gs + c] = L.snd[2 * ls + c];
                    sfd[2 * gs + c] = L.sfd[2 * ls + c];
                }
            }
        }
        for (int64_t x : L.ref_face_slot) s->ref_face_slot.push_back(gslot(x));
        s->ref_nedge.insert(s->ref_nedge.end(), L.ref_nedge.begin(), L.ref_nedge.end());
        for (int64_t x = 0; x < L.Eint; x++) {
            eslot[2 * (e0 + x)] = gslot(L.eslot[2 * x]);
            eslot[2 * (e0 + x) + 1] = gslot(L.eslot[2 * x + 1]);
            ecell[2 * (e0 + x)] = gcell(L.ecell[2 * x]);
            ecell[2 * (e0 + x) + 1] = gcell(L.ecell[2 * x + 1]);
            en[2 * (e0 + x)] = L.en[2 * x];
            en[2 * (e0 + x) + 1] = L.en[2 * x + 1];
            elen[e0 + x] = L.elen[x];
            eref[e0 + x] = L.eref[x];
        }
        for (int64_t b = 0; b < L.G; b++) {
            const int64_t gb = g0 + b;
            bcell[gb] = gcell(L.bcell[b]);
            bslot[gb] = gslot(L.bslot[b]);
            btype[gb] = L.btype[b];
            bref[gb] = L.bref[b];
            bn[2 * gb] = L.bn[2 * b];
            bn[2 * gb + 1] = L.bn[2 * b + 1];
            blen[gb] = L.blen[b];
            for (int c = 0; c < 4; c++) {
                brefl[4 * gb + c] = L.brefl[4 * b + c];
                bdata[4 * gb + c] = L.bdata[4 * b + c];
                bdq[4 * gb + c] = L.bdq[4 * b + c];
                bdmid[4 * gb + c] = L.bdmid[4 * b + c];
            }
            for (int c = 0; c < 8; c++) grad[8 * (Ct + gb) + c] = L.grad[8 * (C + b) + c];
        }
        for (int32_t b : L.force) force.push_back((int32_t)(g0 + b));
        force_off[k + 1] = (int32_t)force.size();
        inst_c0[k + 1] = (int32_t)(c0 + C);
        const int nb = (int)((C + UPD - 1) / UPD);
        for (int b = 0; b < nb; b++) {
            blk_first.push_back((int32_t)(c0 + (int64_t)b * UPD));
            blk_end.push_back((int32_t)(c0 + C));
            blk_inst.push_back(k);
        }
        inst_blk[k + 1] = inst_blk[k] + nb;
        inst_mu[k] = L.mu;
        inst_muf[k] = (float)L.mu;
    }

    s->flux_ref.assign(eref.begin(), eref.end());
    s->flux_ref.insert(s->flux_ref.end(), bref.begin(), bref.end());

    // ---- device allocation (one arena) ----------------------------------------
    const bool split = precision == EBB_PREC_SPLIT;
    const bool dfp = precision == EBB_PREC_DF;
    const int64_t NQ = Ct + Gt;
    const int nblk = D.nblk;
    s->nred = nblk;
    const size_t total = bytes_of(D, precision);
    s->dbytes = total;
    cudaError_t ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaMalloc(&s->dmem, total);
    if (ce != cudaSuccess) {
        e = std::string("CUDA: ") + cudaGetErrorString(ce);
        return ce == cudaErrorMemoryAllocation ? EBB_ERR_OOM : EBB_ERR_CUDA;
    }
    cudaMemsetAsync(s->dmem, 0, total, s->stream);
    Arena ar{(char *)s->dmem, 0, total};
    DArrays &A = s->A;
    auto takeR = [&](size_t m) -> void * { return split ? (void *)ar.take<float>(m) : (void *)ar.take<double>(m); };
    A.q64 = ar.take<double>(4 * NQ);
    A.qs1 = (split || dfp) ? takeR(4 * NQ) : (void *)A.q64;
    A.qs = takeR(4 * NQ);
    A.aux = takeR(4 * NQ);
    A.face = takeR(4 * MJ * Cs);
    A.grad = takeR(8 * NQ);
    A.fl = takeR(4 * (Et + Gt));
    A.fs = takeR(Et + Gt);
    A.cdt = takeR(Ct);
    A.red = ar.take<double>(8 * (size_t)nblk);
    A.st = ar.take<DState>(n);
    A.rec = ar.take<DRecord>(EBB_REC_CAP);
    A.R = A.aux;
    DMesh &M = s->M;
    std::memset(&M, 0, sizeof M);
    M.C = (int32_t)Ct;
    M.G = (int32_t)Gt;
    M.Cs = (int32_t)Cs;
    M.Eint = (int32_t)Et;
    M.maxJ = MJ;
    M.uniform = std::all_of(nedge.begin(), nedge.end(), [&](int32_t v) { return v == MJ; }) ? 1 : 0;
    M.n_inst = n;
    M.n_upd_blocks = nblk;
    auto up = [&](auto *dst, const auto &v) {
        if (!v.empty()) cudaMemcpyAsync((void *)dst, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice, s->stream);
        return dst;
    };
    auto upR = [&](const std::vector<double> &v) -> const void * {
        void *dst = takeR(v.size() ? v.size() : 1);
        if (v.empty()) return dst;
        if (split) {
            std::vector<float> f(v.begin(), v.end());
            cudaMemcpyAsync(dst, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream);
            cudaStreamSynchronize(s->stream);
        } else if (dfp) {
            std::vector<ebbdf::df> f(v.begin(), v.end());
            cudaMemcpyAsync(dst, f.data(), f.size() * sizeof(ebbdf::df), cudaMemcpyHostToDevice, s->stream);
            cudaStreamSynchronize(s->stream);
        } else {
            cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream);
        }
        return dst;
    };
    M.nedge = up(ar.take<int32_t>(Ct), nedge);
    M.cell_ref = up(ar.take<int32_t>(Ct), cellref);
    s->d_perm = up(ar.take<int32_t>(Ct), s->perm);
    {
        std::vector<int32_t> iperm(Ct);
        for (int64_t i = 0; i < Ct; i++) iperm[s->perm[i]] = (int32_t)i;
        s->d_iperm = up(ar.take<int32_t>(Ct), iperm);
    }
    M.g.neg_inv_area = upR(nia);
    M.g.perim = upR(perim);
    M.g.dlen = upR(d);
    M.g.src = any_mms ? upR(src) : nullptr;
    M.s_nbr = up(ar.take<int32_t>(MJ * Cs), snbr);
    M.s_edge = up(ar.take<int32_t>(MJ * Cs), sedge);
    M.g.s_gm = upR(sgm);
    M.g.s_nd = upR(snd);
    M.g.s_fd = upR(sfd);
    M.e_slot = up(ar.take<int32_t>(2 * Et), eslot);
    M.e_cell = up(ar.take<int32_t>(2 * Et), ecell);
    M.g.e_n = upR(en);
    M.g.e_len = upR(elen);
    if (split) {  // per-slot copies for the split update's freestream correction
        std::vector<double> sen(2 * MJ * Cs, 0.0), selen(MJ * Cs, 0.0);
        for (int64_t i = 0; i < Ct; i++)
            for (int j = 0; j < nedge[i]; j++) {
                const int64_t gs = (int64_t)j * Cs + i;
                const int64_t f = sedge[gs] & 0x7fffffff;
                const bool in = f < Et;
                sen[2 * gs] = in ? en[2 * f] : bn[2 * (f - Et)];
                sen[2 * gs + 1] = in ? en[2 * f + 1] : bn[2 * (f - Et) + 1];
                selen[gs] = in ? elen[f] : blen[f - Et];
            }
        M.g.s_en = upR(sen);
        M.g.s_elen = upR(selen);
    } else {
        M.g.s_en = M.g.s_elen = nullptr;
    }
    M.e_ref = up(ar.take<int32_t>(Et), eref);
    M.b_cell = up(ar.take<int32_t>(Gt), bcell);
    M.b_slot = up(ar.take<int32_t>(Gt), bslot);
    M.b_type = up(ar.take<int32_t>(Gt), btype);
    M.b_ref = up(ar.take<int32_t>(Gt), bref);
    M.g.b_n = upR(bn);
    M.g.b_len = upR(blen);
    M.g.b_refl = upR(brefl);
    M.g.b_data = upR(bdata);
    M.g.b_dq = upR(bdq);
    M.g.b_dmid = upR(bdmid);
    M.force_b = up(ar.take<int32_t>(force.size() + 1), force);
    M.n_force = (int32_t)force.size();
    M.force_off = up(ar.take<int32_t>(n + 1), force_off);
    if (n > 1) {
        M.cell_inst = up(ar.take<int32_t>(Ct), cell_inst);
        M.blk_first = up(ar.take<int32_t>(nblk), blk_first);
        M.blk_end = up(ar.take<int32_t>(nblk), blk_end);
        M.blk_inst = up(ar.take<int32_t>(nblk), blk_inst);
        M.inst_blk = up(ar.take<int32_t>(n + 1), inst_blk);
        M.inst_c0 = up(ar.take<int32_t>(n + 1), inst_c0);
        M.inst_mu = up(ar.take<double>(n), inst_mu);
        M.inst_muf = up(ar.take<float>(n), inst_muf);
    }
    s->d_stage = ar.take<double>(4 * Ct);
    s->d_tmp = ar.take<double>(4 * Ct);
    up(A.q64, q);
    if (split) {
        std::vector<float> gf(grad.begin(), grad.end());
        cudaMemcpyAsync(A.grad, gf.data(), gf.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream);
        cudaStreamSynchronize(s->stream);
        launch_to_float4(A.q64, reinterpret_cast<float *>(A.qs1), Ct, s->stream);
    } else if (dfp) {
        std::vector<ebbdf::df> gw(grad.begin(), grad.end());
        cudaMemcpyAsync(A.grad, gw.data(), gw.size() * sizeof(ebbdf::df), cudaMemcpyHostToDevice, s->stream);
        cudaStreamSynchronize(s->stream);
        launch_to_df4(A.q64, A.qs1, Ct, s->stream);
    } else {
        up(reinterpret_cast<double *>(A.grad), grad);
    }
    const ebb_config &c0 = Ls[0].cfg;
    DPhys &P = s->P;
    P.flux = c0.flux;
    P.limited = c0.limited;
    P.order = (int32_t)c0.order;
    P.viscous = c0.viscosity;
    P.mms = c0.mms;
    P.local_ts = c0.local_timestep;
    P.lp = (c0.lp_thresh > 0) ? 1 : 0;
    P.lp_thresh = c0.lp_thresh;
    P.pr = c0.pr;
    P.mu = Ls[0].mu;
    P.prf = (float)P.pr;
    P.muf = (float)P.mu;
    // the same IEEE double operations the viscous flux (flux.d:28-64) performs per face
    P.gP = 1.4 / P.pr;
    P.c43gP = (-4.0 / 3.0) + P.gP;
    P.m1gP = -1.0 + P.gP;
    P.p43mgP = (4.0 / 3.0) - P.gP;
    P.omgP = 1.0 - P.gP;
    P.gPw = P.gP;
    P.c43gPw = P.c43gP;
    P.m1gPw = P.m1gP;
    P.p43mgPw = P.p43mgP;
    P.omgPw = P.omgP;
    P.muw = P.mu;
    P.r_gas = c0.r_gas;
    P.need_grad = (c0.viscosity || visc_wall) ? 1 : 0;
    std::vector<DState> st(n);
    for (int k = 0; k < n; k++) {
        st[k] = Ls[k].st0;
        st[k].rec_enabled = n == 1;
    }
    cudaMemcpyAsync(A.st, st.data(), sizeof(DState) * n, cudaMemcpyHostToDevice, s->stream);
    ce = cudaStreamSynchronize(s->stream);
    if (ce != cudaSuccess) {
        e = std::string("CUDA: ") + cudaGetErrorString(ce);
        return EBB_ERR_CUDA;
    }
    return EBB_OK;
}

}  // namespace ebb
