// solver_impl.hpp -- the solver handle behind the C ABI (host side).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "host.hpp"
#include "layout.h"

namespace ebb {

// One mesh + config laid out in local numbering (cells 0..C-1, ghosts C..C+G-1,
// interior edges 0..Eint-1 then boundary edges, ELL slot (i, j) at j*C + i).
struct InstLayout {
    ebb_config cfg;
    int64_t C = 0, G = 0, Eint = 0;
    int maxJ = 0;
    double mu = 0;
    bool any_visc_wall = false;
    std::vector<int32_t> perm, cellref, nedge, snbr, sedge, eslot, ecell, eref;
    std::vector<int32_t> bcell, bslot, btype, bref, force, ref_nedge;
    std::vector<int64_t> ref_face_slot;
    std::vector<double> nia, perim, d, src, sgm, snd, sfd, en, elen, bn, blen, brefl, bdata, bdq, bdmid, grad, q;
    DState st0;
};

// Where an instance sits in the arena.
struct InstMeta {
    int64_t c0 = 0, C = 0, g0 = 0, G = 0, e0 = 0, Eint = 0;
    ebb_config cfg;
};

}  // namespace ebb

struct ebb_solver {
    ebb_config cfg;
    int32_t n_inst = 1;
    std::vector<ebb::InstMeta> inst;
    int32_t precision = EBB_PREC_FP64;
    int64_t C = 0, G = 0, Eint = 0, Cs = 0;
    int32_t maxJ = 0;
    double mu = 0;
    std::vector<int32_t> perm;           // device cell -> reference cell
    std::vector<int64_t> ref_face_slot;  // reference (cell, local edge) order -> device slot index
    std::vector<int32_t> ref_nedge;      // edge count per reference cell
    std::vector<int32_t> flux_ref;       // flux index (interior edges, then boundary) -> reference edge id
    cudaStream_t stream = nullptr;
    void *dmem = nullptr;
    size_t dbytes = 0;
    DMesh M{};
    DPhys P{};
    DArrays A{};
    int32_t *d_perm = nullptr;
    int32_t *d_iperm = nullptr;  // reference cell -> device cell
    double *d_stage = nullptr;  // C x 4 doubles in reference order
    double *d_tmp = nullptr;    // C x 4 doubles in device order (split-path conversions)
    int nred = 0;
    cudaGraphExec_t g1 = nullptr, g16 = nullptr;  // 1-step and 16-step time-loop graphs
    int32_t err_kind = 0;
    int64_t err_index = -1;
    std::string err_msg;
};

namespace ebb {
int solver_sync_state(ebb_solver *s, DState &hst);
int solver_write_state(ebb_solver *s, const DState &hst);
int solver_sync_all(ebb_solver *s, std::vector<DState> &h);
int solver_write_all(ebb_solver *s, const std::vector<DState> &h);
int solver_run_residual_on_qs(ebb_solver *s, int limit, int dt_update, double *new_dt, double *rmax);
int build_instance(const ebb_mesh *mesh, const ebb_config *cfg, InstLayout &L, std::string &err);
int assemble(ebb_solver *s, std::vector<InstLayout> &layouts, int32_t precision, std::string &err);
size_t arena_bytes(const std::vector<InstLayout> &layouts, int32_t precision);
int read_esln_into(const char *path, std::vector<double> &q, std::vector<uint8_t> &seen, double &t, double &dt);
int write_esln_points(const char *path, int64_t n, const double *q, double t, double dt, uint32_t order);
}  // namespace ebb
