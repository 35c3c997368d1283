// reconstruct.cpp -- ebb-reconstruct (app/reconstruct.d:79-424) on the GPU.
//
// One residual evaluation of the resident state (limited as config.limited, no time
// step update: stepMesh, reconstruct.d:79-176) leaves the face states of every edge;
// with the limiter values exported by k_cell and the raw gradients, the device then
// computes the edge values (mean of an edge's two states) and the node values
// (gradient extrapolation averaged over a node's cells; boundary nodes average their
// boundary edges).  The host assembles the refined triangulation -- the nodes the
// elements use, the edge midpoints and the cell centroids as points, each cell split
// into 2 x nEdges triangles -- and writes it as .mmsh (saveMatlabMesh, io.d:534-643)
// and .esln (saveSolution of points without edges, reconstruct.d:416-420).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "solver_impl.hpp"

using namespace ebb;

namespace {

struct BEW {
    std::vector<uint8_t> b;
    void u64(uint64_t v)
    {
        for (int k = 7; k >= 0; k--) b.push_back((uint8_t)(v >> (8 * k)));
    }
    void f64(double d)
    {
        uint64_t v;
        std::memcpy(&v, &d, 8);
        u64(v);
    }
};

// The refined mesh of reconstruct.d:240-414 (node numbers 1-based).
struct Refined {
    std::vector<int32_t> used;       // original node id of each used node, node order
    std::vector<int32_t> node_map;   // original node -> 1-based used-node number, or 0
    std::vector<uint8_t> is_b;       // per used node
    std::vector<int32_t> off, items; // per used node: device cells, or reference boundary edges
    std::vector<double> nxy;         // per used node
    std::vector<double> pts;         // used nodes, edge midpoints, centroids (x, y)
    std::vector<double> tris;        // 3 node numbers per triangle (as the .mmsh stores them)
};

int build_refined(const ebb_mesh &m, const Topology &t, const std::vector<int32_t> &inv_perm, Refined &R)
{
    const int64_t N = (int64_t)m.xy.size() / 2, C = t.C, E = t.E;
    const int64_t ne = (int64_t)m.elem_off.size() - 1;
    if (ne != C) return EBB_ERR_MESH;
    std::vector<int32_t> cnt(N + 1, 0);
    for (int64_t c = 0; c < C; c++)
        for (int64_t k = m.elem_off[c]; k < m.elem_off[c + 1]; k++) cnt[m.elem_nodes[k] + 1]++;
    for (int64_t n = 0; n < N; n++) cnt[n + 1] += cnt[n];
    std::vector<int32_t> cells(cnt[N]), fill(N, 0);
    for (int64_t c = 0; c < C; c++)  // ascending element order per node
        for (int64_t k = m.elem_off[c]; k < m.elem_off[c + 1]; k++) {
            const int32_t n = m.elem_nodes[k];
            cells[cnt[n] + fill[n]++] = (int32_t)c;
        }
    std::vector<uint8_t> bnode(N, 0);
    for (size_t b = 0; 2 * b + 1 < m.b_nodes.size(); b++) {
        bnode[m.b_nodes[2 * b]] = 1;
        bnode[m.b_nodes[2 * b + 1]] = 1;
    }
    R.node_map.assign(N, 0);
    R.off.assign(1, 0);
    for (int64_t n = 0; n < N; n++) {
        if (cnt[n + 1] == cnt[n]) continue;  // orphaned node (reconstruct.d:247-268)
        R.used.push_back((int32_t)n);
        R.node_map[n] = (int32_t)R.used.size();
        R.is_b.push_back(bnode[n]);
        R.nxy.push_back(m.xy[2 * n]);
        R.nxy.push_back(m.xy[2 * n + 1]);
        for (int32_t a = cnt[n]; a < cnt[n + 1]; a++) {
            const int32_t c = cells[a];
            if (!bnode[n]) {
                R.items.push_back(inv_perm[c]);
                continue;
            }
            const int nE = t.nedge[c];
            for (int j = 0; j < nE; j++) {
                const int32_t n1 = m.elem_nodes[m.elem_off[c] + j];
                const int32_t n2 = m.elem_nodes[m.elem_off[c] + (j + 1) % nE];
                const int32_t e = t.slot_edge[(int64_t)c * kMaxEdges + j];
                if (t.e_boundary[e] && (n1 == n || n2 == n)) R.items.push_back(e);
            }
        }
        R.off.push_back((int32_t)R.items.size());
    }
    const int64_t nU = (int64_t)R.used.size();
    R.pts.reserve(2 * (nU + E + C));
    R.pts.insert(R.pts.end(), R.nxy.begin(), R.nxy.end());
    for (int64_t e = 0; e < E; e++) {
        R.pts.push_back(t.e_mx[e]);
        R.pts.push_back(t.e_my[e]);
    }
    for (int64_t c = 0; c < C; c++) {
        R.pts.push_back(t.cx[c]);
        R.pts.push_back(t.cy[c]);
    }
    for (int64_t c = 0; c < C; c++) {  // reconstruct.d:380-399
        const int nE = t.nedge[c];
        const double cn = (double)(nU + E + c + 1);
        for (int j = 0; j < nE; j++) {
            const double n1 = R.node_map[m.elem_nodes[m.elem_off[c] + j]];
            const double n2 = R.node_map[m.elem_nodes[m.elem_off[c] + (j + 1) % nE]];
            const double en = (double)(nU + t.slot_edge[c * kMaxEdges + j] + 1);
            const double tri[6] = {n1, en, cn, en, n2, cn};
            R.tris.insert(R.tris.end(), tri, tri + 6);
        }
    }
    return EBB_OK;
}

// saveMatlabMesh (io.d:534-643) of the refined mesh: it has no edges and no tags
int write_mmsh(const char *path, const Refined &R)
{
    BEW w;
    const uint64_t np = R.pts.size() / 2, nt = R.tris.size() / 3;
    w.b.reserve(40 + 8 * (R.pts.size() + R.tris.size()));
    w.u64(np);
    for (double v : R.pts) w.f64(v);
    w.u64(nt);
    for (double v : R.tris) w.f64(v);
    w.u64(0);  // interior edges
    w.u64(0);  // boundary edges
    w.u64(0);  // boundary tags
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return EBB_ERR_IO;
    const size_t n = std::fwrite(w.b.data(), 1, w.b.size(), fp);
    std::fclose(fp);
    return n == w.b.size() ? EBB_OK : EBB_ERR_IO;
}

}  // namespace

extern "C" {

int ebb_reconstruct(ebb_solver *s, const ebb_mesh *mesh, const char *mmsh_path, const char *esln_path, double t,
                    double dt, double *q_out, int64_t *n_out)
{
    if (!s || !mesh) return EBB_ERR_ARG;
    if (s->n_inst != 1) return EBB_ERR_ARG;
    Topology topo;
    std::string e;
    if (!build_topology(*mesh, topo, e) || topo.C != s->C || topo.E != s->Eint + s->G) return EBB_ERR_MESH;
    std::vector<int32_t> inv(s->C);
    for (int64_t k = 0; k < s->C; k++) inv[s->perm[k]] = (int32_t)k;
    Refined R;
    int r = build_refined(*mesh, topo, inv, R);
    if (r) return r;
    const int64_t nU = (int64_t)R.used.size(), E = topo.E, C = s->C, n_all = nU + E + C;
    if (n_out) *n_out = n_all;
    if (!q_out && !mmsh_path && !esln_path) return EBB_OK;  // size query

    // device buffers of the reconstruction (post-processing: allocated per call)
    const bool split = s->precision == EBB_PREC_SPLIT, dfp = s->precision == EBB_PREC_DF;
    const size_t rs = split ? sizeof(float) : sizeof(double);  // a double-float is 8 bytes
    std::vector<double> cxy(2 * C);
    for (int64_t i = 0; i < C; i++) {  // centroids in device cell order
        cxy[2 * i] = topo.cx[s->perm[i]];
        cxy[2 * i + 1] = topo.cy[s->perm[i]];
    }
    const size_t b_lim = 8 * C * rs, b_edge = 4 * E * sizeof(double), b_node = 4 * nU * sizeof(double);
    const size_t b_off = (nU + 1) * sizeof(int32_t), b_items = (R.items.size() + 1) * sizeof(int32_t);
    const size_t b_isb = nU + 1, b_nxy = 2 * nU * sizeof(double) + 8, b_cxy = 2 * C * sizeof(double);
    size_t parts[] = {b_lim, b_edge, b_node, b_off, b_items, b_isb, b_nxy, b_cxy, sizeof(unsigned long long)};
    size_t total = 0, offs[9];
    for (int k = 0; k < 9; k++) {
        offs[k] = total;
        total += (parts[k] + 255) & ~(size_t)255;
    }
    char *d = nullptr;
    if (cudaMalloc(&d, total) != cudaSuccess) return EBB_ERR_OOM;
    auto P_ = [&](int k) { return d + offs[k]; };
    cudaStream_t st = s->stream;
    cudaMemcpyAsync(P_(3), R.off.data(), R.off.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (!R.items.empty())
        cudaMemcpyAsync(P_(4), R.items.data(), R.items.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (nU) cudaMemcpyAsync(P_(5), R.is_b.data(), nU, cudaMemcpyHostToDevice, st);
    if (nU) cudaMemcpyAsync(P_(6), R.nxy.data(), 2 * nU * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(P_(7), cxy.data(), b_cxy, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(P_(8), 0xff, sizeof(unsigned long long), st);

    // stepMesh: one evaluation on the resident state with gradients and limiters kept
    if (split)
        launch_to_float4(s->A.q64, reinterpret_cast<float *>(s->A.qs), C, st);
    else if (dfp)
        launch_to_df4(s->A.q64, s->A.qs, C, st);
    else
        cudaMemcpyAsync(s->A.qs, s->A.q64, 4 * C * sizeof(double), cudaMemcpyDeviceToDevice, st);
    const int32_t need_grad = s->P.need_grad;
    s->P.need_grad = 1;
    s->A.lim = P_(0);
    double new_dt = 0, rmax = 0;
    r = solver_run_residual_on_qs(s, s->cfg.limited, 0, &new_dt, &rmax);
    if (r == EBB_OK) {
        r = split ? launch_recon<float>(s->M, s->A, reinterpret_cast<const float *>(s->A.qs), (double *)P_(1), (int)nU,
                                        (const int32_t *)P_(3), (const int32_t *)P_(4), (const uint8_t *)P_(5),
                                        (const double *)P_(6), (const double *)P_(7), (double *)P_(2),
                                        (unsigned long long *)P_(8), st)
            : dfp ? launch_recon<ebbdf::df>(s->M, s->A, reinterpret_cast<const ebbdf::df *>(s->A.qs), (double *)P_(1),
                                            (int)nU, (const int32_t *)P_(3), (const int32_t *)P_(4),
                                            (const uint8_t *)P_(5), (const double *)P_(6), (const double *)P_(7),
                                            (double *)P_(2), (unsigned long long *)P_(8), st)
                  : launch_recon<double>(s->M, s->A, reinterpret_cast<const double *>(s->A.qs), (double *)P_(1),
                                         (int)nU, (const int32_t *)P_(3), (const int32_t *)P_(4),
                                         (const uint8_t *)P_(5), (const double *)P_(6), (const double *)P_(7),
                                         (double *)P_(2), (unsigned long long *)P_(8), st);
        r = r ? EBB_ERR_CUDA : EBB_OK;
    }
    s->A.lim = nullptr;
    s->P.need_grad = need_grad;
    std::vector<double> vals(4 * n_all);
    unsigned long long bad = ~0ull;
    if (r == EBB_OK) {
        cudaMemcpyAsync(vals.data(), P_(2), b_node, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(vals.data() + 4 * nU, P_(1), b_edge, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&bad, P_(8), sizeof bad, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) r = EBB_ERR_CUDA;
    }
    cudaFree(d);
    if (r) return r;
    if (bad != ~0ull) {  // reconstruct.d:320-322,344-346: NaN node value
        s->err_kind = EBB_ERR_NAN_CELL;
        s->err_index = (int64_t)bad;
        s->err_msg = "New node value is NaN";
        return EBB_ERR_NAN_CELL;
    }
    if ((r = ebb_get_state(s, vals.data() + 4 * (nU + E)))) return r;
    if (q_out) std::memcpy(q_out, vals.data(), vals.size() * sizeof(double));
    if (mmsh_path && (r = write_mmsh(mmsh_path, R))) return r;
    if (esln_path && (r = write_esln_points(esln_path, n_all, vals.data(), t, dt, (uint32_t)s->cfg.order))) return r;
    return EBB_OK;
}

}  // extern "C"
