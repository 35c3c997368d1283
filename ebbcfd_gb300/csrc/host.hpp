// host.hpp -- host-side data structures of the GB300 solver library.
//
// The host keeps the reference's mesh semantics (gmsh reader of source/io.d:689-990,
// buildMesh of source/mesh.d:217-643) and turns them into the device layout:
// Hilbert-ordered cells, ELL ("slot-major") per-face arrays, edge lists sorted by
// their first cell, all precomputed in FP64.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ebb_gb300.h"

struct ebb_mesh {
    std::vector<double> xy;            // 2 * n_nodes
    std::vector<int64_t> elem_off;     // n_elem + 1
    std::vector<int32_t> elem_nodes;   // 0-based node ids, counter-clockwise
    std::vector<int32_t> b_nodes;      // 2 * n_b, 0-based
    std::vector<int64_t> b_group_start;
    std::vector<std::string> tags;
    int32_t max_edges = 0;
};

namespace ebb {

constexpr int kMaxEdges = 6;

void set_err(char *err, size_t len, const std::string &msg);

// Topology and FP64 geometry in reference numbering (mesh.d:217-643).
struct Topology {
    int64_t C = 0;                  // interior cells
    int64_t G = 0;                  // boundary edges == ghost cells (creation order)
    int64_t E = 0;                  // edges (interior + boundary)
    int32_t maxJ = 0;               // largest element edge count
    // per cell
    std::vector<int32_t> nedge;
    std::vector<double> area, perim, d, cx, cy;
    // per face slot (cell i, local edge j) at i*kMaxEdges + j
    std::vector<int32_t> slot_edge;  // edge id
    std::vector<int8_t> slot_sign;   // fluxMultiplier (+1 / -1)
    std::vector<int32_t> slot_nbr;   // neighbour cell (interior id, or C + ghost id)
    std::vector<double> gm0, gm1;    // gradMat rows, per slot
    // per edge
    std::vector<int32_t> e_cell0, e_cell1;  // cellIdx[0] (creator), cellIdx[1] (other or C + ghost)
    std::vector<double> e_len, e_nx, e_ny, e_mx, e_my;
    std::vector<int32_t> e_node0, e_node1;  // creator orientation
    std::vector<int8_t> e_boundary;
    std::vector<int32_t> e_group;           // boundary group (tag index) or -1
    // per ghost (boundary edge in creation order)
    std::vector<int32_t> g_edge;            // edge id
    std::vector<double> g_cx, g_cy;         // reflected centroid
};

bool build_topology(const ebb_mesh &m, Topology &t, std::string &err);

// Hilbert-curve order of the cell centroids: perm[new] = old.
std::vector<int32_t> hilbert_order(const Topology &t);

// JSON
bool parse_config_json(const char *text, ebb_config *out, std::string &err);

// manufactured solutions (host FP64)
void mms_solution(int kind, double x, double y, double q[4]);
void mms_gradient(int kind, double x, double y, double g[4][2]);
void mms_source(int kind, double x, double y, const ebb_config &cfg, double mu, double S[4]);

}  // namespace ebb
