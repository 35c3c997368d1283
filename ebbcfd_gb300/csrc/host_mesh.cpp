// host_mesh.cpp -- gmsh 2.2 reader, topology/geometry build and the cell ordering.
//
// Reader semantics follow source/io.d:689-990 (parseGmshMesh); topology and FP64
// geometry follow source/mesh.d:217-381,481-642 (UMesh2.buildMesh).  The design is
// this library's own: one pass over a memory-mapped token stream, sort-based edge
// matching instead of a sparse hash, and flat arrays instead of per-cell structs.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <unordered_map>

#include "host.hpp"

namespace ebb {

void set_err(char *err, size_t len, const std::string &msg)
{
    if (err && len) {
        size_t n = std::min(len - 1, msg.size());
        std::memcpy(err, msg.data(), n);
        err[n] = 0;
    }
}

namespace {

struct LineReader {
    const char *p, *end;
    explicit LineReader(const std::string &s) : p(s.data()), end(s.data() + s.size()) {}
    bool eof() const { return p >= end; }
    // next line split on blanks/tabs (io.d:662-666: strip, detab, split(' '), drop empties)
    std::vector<std::string> tokens()
    {
        std::vector<std::string> out;
        const char *q = p;
        while (q < end && *q != '\n') q++;
        const char *s = p;
        p = (q < end) ? q + 1 : end;
        while (s < q) {
            while (s < q && (*s == ' ' || *s == '\t' || *s == '\r' || *s == '\v' || *s == '\f')) s++;
            const char *t = s;
            while (t < q && !(*t == ' ' || *t == '\t' || *t == '\r' || *t == '\v' || *t == '\f')) t++;
            if (t > s) out.emplace_back(s, t - s);
            s = t;
        }
        return out;
    }
    // fast path for numeric lines: parse up to n numbers into vals, return count
    int numbers(double *vals, int n, bool &ok)
    {
        const char *q = p;
        while (q < end && *q != '\n') q++;
        std::string line(p, q - p);
        p = (q < end) ? q + 1 : end;
        const char *s = line.c_str();
        int k = 0;
        ok = true;
        while (*s) {
            while (*s == ' ' || *s == '\t' || *s == '\r') s++;
            if (!*s) break;
            char *e;
            double v = std::strtod(s, &e);
            if (e == s) {
                ok = false;
                return k;
            }
            if (k < n) vals[k] = v;
            k++;
            s = e;
        }
        return k;
    }
};

bool to_int(const std::string &s, long long &v)
{
    if (s.empty()) return false;
    char *e;
    v = std::strtoll(s.c_str(), &e, 10);
    return *e == 0;
}

// ebb.math.sum over ".length" (source/math.d:18-33): for lists longer than 6 the
// recursion drops elements m-1 and the last one.  Kept because the boundary-group
// bookkeeping of io.d:918-955 depends on it.
int64_t ebb_sum_lengths(const std::vector<int64_t> &d, size_t lo, size_t hi)
{
    size_t n = hi - lo;
    if (n <= 6) {
        int64_t s = d[lo];
        for (size_t i = lo + 1; i < hi; i++) s += d[i];
        return s;
    }
    size_t m = (size_t)std::floor((double)n / 2.0);
    return ebb_sum_lengths(d, lo, lo + m - 1) + ebb_sum_lengths(d, lo + m, hi - 1);
}

int64_t sum_group_lengths(const std::vector<std::vector<int32_t>> &g, size_t count)
{
    if (count == 0) return 0;
    std::vector<int64_t> lens(count);
    for (size_t i = 0; i < count; i++) lens[i] = (int64_t)g[i].size();
    return ebb_sum_lengths(lens, 0, count);
}

}  // namespace

bool read_gmsh(const std::string &path, ebb_mesh &m, std::string &err)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        err = "cannot open mesh file " + path;
        return false;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    std::string text = ss.str();
    LineReader r(text);

    std::vector<std::vector<int32_t>> bGroups;  // tag id per line element, split where the tag changes
    std::vector<int32_t> bNodes;                 // pairs
    std::vector<int32_t> elNodes;
    std::vector<int64_t> elOff{0};
    std::vector<double> xy;

    auto end_section = [&]() -> bool {
        auto t = r.tokens();
        if (t.empty() || t[0].find("$End") == std::string::npos) {
            err = "Expected section end";
            return false;
        }
        return true;
    };

    while (!r.eof()) {
        auto t = r.tokens();
        while (t.empty() && !r.eof()) t = r.tokens();
        if (t.empty()) break;
        if (t.size() != 1 || t[0][0] != '$') {
            err = "Incorrectly formatted section header";
            return false;
        }
        std::string sec = t[0].substr(1);
        if (sec == "MeshFormat") {
            auto fl = r.tokens();
            long long fmt;
            if (fl.size() < 2 || !to_int(fl[1], fmt) || fmt != 0) {
                err = "Unsuported mesh format. Expected 0";
                return false;
            }
            if (!end_section()) return false;
        } else if (sec == "PhysicalNames") {
            auto nl = r.tokens();
            long long n;
            if (nl.size() != 1 || !to_int(nl[0], n)) {
                err = "Unexpected number of entries in PhysicalNames";
                return false;
            }
            for (long long i = 0; i < n; i++) {
                if (r.eof()) {
                    err = "Unexpected end of file";
                    return false;
                }
                auto l = r.tokens();
                long long dim;
                if (l.size() != 3 || !to_int(l[0], dim)) {
                    err = "Expected 3 entries in a PhysicalNames line";
                    return false;
                }
                if (dim == 1) {
                    std::string s = l[2];
                    size_t a = 0, b = s.size();
                    while (a < b && s[a] == '"') a++;
                    while (b > a && s[b - 1] == '"') b--;
                    m.tags.push_back(s.substr(a, b - a));
                }
            }
            if (!end_section()) return false;
        } else if (sec == "Nodes") {
            auto nl = r.tokens();
            long long n;
            if (nl.size() != 1 || !to_int(nl[0], n) || n < 0) {
                err = "Unexpected number of entries in Nodes";
                return false;
            }
            xy.resize(2 * (size_t)n);
            for (long long i = 0; i < n; i++) {
                if (r.eof()) {
                    err = "Unexpected end of file";
                    return false;
                }
                double v[8];
                bool ok;
                int k = r.numbers(v, 8, ok);
                if (!ok || k < 4 || (long long)v[0] != i + 1) {
                    err = "Unexpected node line " + std::to_string(i + 1);
                    return false;
                }
                xy[2 * i] = v[1];
                xy[2 * i + 1] = v[2];
            }
            if (!end_section()) return false;
        } else if (sec == "Elements") {
            auto nl = r.tokens();
            long long n;
            if (nl.size() != 1 || !to_int(nl[0], n) || n < 0) {
                err = "Unexpected number of entries in Elements";
                return false;
            }
            int32_t cur = -1;
            for (long long i = 0; i < n; i++) {
                if (r.eof()) {
                    err = "Unexpected end of file";
                    return false;
                }
                double v[64];
                bool ok;
                int k = r.numbers(v, 64, ok);
                if (!ok || k <= 4 || k > 64) {
                    err = "Element line must have at least 4 entries";
                    return false;
                }
                if ((long long)v[0] != i + 1) {
                    err = "Unexpected element number " + std::to_string(i + 1);
                    return false;
                }
                int type = (int)v[1], ntags = (int)v[2];
                if (ntags < 1 || 3 + ntags > k) {
                    err = "Expected at least one element tag";
                    return false;
                }
                if (type == 1) {
                    int32_t g = (int32_t)v[3];
                    if (k - (3 + ntags) != 2) {
                        err = "line element needs two nodes";
                        return false;
                    }
                    if (g != cur) {
                        cur = g;
                        bGroups.emplace_back();
                    }
                    bGroups.back().push_back(g);
                    bNodes.push_back((int32_t)v[3 + ntags] - 1);
                    bNodes.push_back((int32_t)v[4 + ntags] - 1);
                } else if (type == 2 || type == 3) {
                    int nn = k - (3 + ntags);
                    if (nn != type + 1) {
                        err = "element node count does not match its type";
                        return false;
                    }
                    for (int j = 0; j < nn; j++) elNodes.push_back((int32_t)v[3 + ntags + j] - 1);
                    elOff.push_back((int64_t)elNodes.size());
                } else {
                    err = "Unsuported element type: " + std::to_string(type);
                    return false;
                }
            }
            if (!end_section()) return false;
        } else {
            for (;;) {
                if (r.eof()) {
                    err = "Unexpected end of file";
                    return false;
                }
                auto l = r.tokens();
                if (!l.empty() && l[0].find("$End") != std::string::npos) break;
            }
        }
    }

    // merge boundary groups that were split in the file (io.d:910-942)
    size_t nB = bNodes.size() / 2;
    if (bGroups.size() != m.tags.size()) {
        std::vector<std::vector<int32_t>> ng;
        std::vector<int32_t> nb;  // pairs
        for (size_t i = 0; i < bGroups.size(); i++) {
            int32_t curg = bGroups[i][0];
            long old = -1;
            for (size_t k = 0; k < ng.size(); k++)
                if (ng[k][0] == curg) {
                    old = (long)k;
                    break;
                }
            int64_t ns = i == 0 ? 0 : sum_group_lengths(bGroups, i);
            int64_t ne = sum_group_lengths(bGroups, i + 1);
            if (ne > (int64_t)nB || ns >= (int64_t)nB || ns < 0 || ne < ns) {
                err = "Computed boundary node index is out of bounds";
                return false;
            }
            if (old >= 0) {
                int64_t nne = sum_group_lengths(ng, (size_t)old + 1);
                if (nne < 0 || 2 * nne > (int64_t)nb.size()) {
                    err = "Computed boundary node index is out of bounds";
                    return false;
                }
                ng[old].insert(ng[old].end(), bGroups[i].begin(), bGroups[i].end());
                std::vector<int32_t> merged(nb.begin(), nb.begin() + 2 * nne);
                merged.insert(merged.end(), bNodes.begin() + 2 * ns, bNodes.begin() + 2 * ne);
                merged.insert(merged.end(), nb.begin() + 2 * nne, nb.end());
                nb.swap(merged);
            } else {
                ng.push_back(bGroups[i]);
                nb.insert(nb.end(), bNodes.begin() + 2 * ns, bNodes.begin() + 2 * ne);
            }
        }
        if (nb.size() != bNodes.size()) {
            err = "Reordered boundary node array length does not match old boundary node array";
            return false;
        }
        bNodes.swap(nb);
        bGroups.swap(ng);
    }
    if (bGroups.size() != m.tags.size()) {
        err = "Number of boundary groups does not match the number of boundary tags";
        return false;
    }
    // reorder boundary nodes by physical tag 1..N (io.d:946-960)
    nB = bNodes.size() / 2;
    for (size_t i = 0; i < bGroups.size(); i++) {
        long gi = -1;
        for (size_t k = 0; k < bGroups.size(); k++)
            if (bGroups[k][0] == (int32_t)(i + 1)) {
                gi = (long)k;
                break;
            }
        if (gi < 0) {
            err = "Could not determine boundary group";
            return false;
        }
        int64_t ne = sum_group_lengths(bGroups, (size_t)gi + 1);
        int64_t ns = gi == 0 ? 0 : sum_group_lengths(bGroups, (size_t)gi);
        if (ne > (int64_t)nB || ns >= (int64_t)nB || ns < 0 || ne < ns) {
            err = "Computed boundary node index is out of bounds";
            return false;
        }
        m.b_group_start.push_back((int64_t)m.b_nodes.size() / 2);
        m.b_nodes.insert(m.b_nodes.end(), bNodes.begin() + 2 * ns, bNodes.begin() + 2 * ne);
    }

    m.xy.swap(xy);
    m.elem_off.swap(elOff);
    m.elem_nodes.swap(elNodes);
    int64_t nn = (int64_t)m.xy.size() / 2;
    for (int32_t v : m.elem_nodes)
        if (v < 0 || v >= nn) {
            err = "element references a missing node";
            return false;
        }
    for (int32_t v : m.b_nodes)
        if (v < 0 || v >= nn) {
            err = "line element references a missing node";
            return false;
        }
    return true;
}

// clockwise elements are reversed (io.d:969-987); max edge count recorded
bool finish_mesh(ebb_mesh &m, std::string &err)
{
    int64_t ne = (int64_t)m.elem_off.size() - 1;
    m.max_edges = 0;
    for (int64_t i = 0; i < ne; i++) {
        int64_t a = m.elem_off[i], b = m.elem_off[i + 1];
        int n = (int)(b - a);
        if (n < 3 || n > kMaxEdges) {
            err = "element " + std::to_string(i) + " has an unsupported number of edges";
            return false;
        }
        m.max_edges = std::max(m.max_edges, n);
        double area = 0;
        for (int j = 0; j < n; j++) {
            int32_t n1 = m.elem_nodes[a + j], n2 = m.elem_nodes[a + (j + 1) % n];
            area += m.xy[2 * n1] * m.xy[2 * n2 + 1] - m.xy[2 * n2] * m.xy[2 * n1 + 1];
        }
        if (area < 0) std::reverse(m.elem_nodes.begin() + a, m.elem_nodes.begin() + b);
    }
    return true;
}

static inline uint64_t pair_key(int32_t a, int32_t b)
{
    uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
    return ((uint64_t)lo << 32) | hi;
}

bool build_topology(const ebb_mesh &m, Topology &t, std::string &err)
{
    const int64_t C = (int64_t)m.elem_off.size() - 1;
    const int K = kMaxEdges;
    t.C = C;
    t.maxJ = m.max_edges;
    t.nedge.assign(C, 0);
    t.area.assign(C, 0.0);
    t.perim.assign(C, 0.0);
    t.d.assign(C, 0.0);
    t.cx.assign(C, 0.0);
    t.cy.assign(C, 0.0);
    t.slot_edge.assign(C * K, -1);
    t.slot_sign.assign(C * K, 1);
    t.slot_nbr.assign(C * K, -1);
    t.gm0.assign(C * K, 0.0);
    t.gm1.assign(C * K, 0.0);

    // boundary membership: sorted node pair -> last line element with that pair (mesh.d:223-228)
    std::unordered_map<uint64_t, int64_t> bmap;
    bmap.reserve(m.b_nodes.size());
    int64_t nB = (int64_t)m.b_nodes.size() / 2;
    for (int64_t i = 0; i < nB; i++) bmap[pair_key(m.b_nodes[2 * i], m.b_nodes[2 * i + 1])] = i;
    const int64_t nGroups = (int64_t)m.b_group_start.size();

    // classify slots; non-boundary slots are matched by sorting (key, slot)
    std::vector<std::pair<uint64_t, int64_t>> keys;
    keys.reserve((size_t)m.elem_nodes.size());
    std::vector<int64_t> slot_bline(C * K, -1);
    for (int64_t i = 0; i < C; i++) {
        int64_t a = m.elem_off[i];
        int n = (int)(m.elem_off[i + 1] - a);
        t.nedge[i] = n;
        for (int j = 0; j < n; j++) {
            int32_t n0 = m.elem_nodes[a + j], n1 = m.elem_nodes[a + (j + 1) % n];
            uint64_t k = pair_key(n0, n1);
            auto it = bmap.find(k);
            if (it != bmap.end())
                slot_bline[i * K + j] = it->second;
            else
                keys.emplace_back(k, i * K + j);
        }
    }
    std::sort(keys.begin(), keys.end());
    // partner slot of each non-boundary slot; the lower slot (earlier element) creates the edge
    std::vector<int64_t> partner(C * K, -1);
    for (size_t s = 0; s < keys.size();) {
        size_t e = s;
        while (e < keys.size() && keys[e].first == keys[s].first) e++;
        if (e - s != 2) {
            int64_t sl = keys[s].second;
            err = (e - s == 1 ? "edge of element " + std::to_string(sl / K) +
                                    " is shared by no other element and is not tagged as boundary"
                              : "edge of element " + std::to_string(sl / K) + " is shared by more than two elements");
            return false;
        }
        partner[keys[s].second] = keys[s + 1].second;
        partner[keys[s + 1].second] = keys[s].second;
        s = e;
    }
    keys.clear();
    keys.shrink_to_fit();

    // create edges in the reference's creation order (element-major, local edge order)
    auto X = [&](int32_t n) { return m.xy[2 * n]; };
    auto Y = [&](int32_t n) { return m.xy[2 * n + 1]; };
    for (int64_t i = 0; i < C; i++) {
        int64_t a = m.elem_off[i];
        int n = t.nedge[i];
        for (int j = 0; j < n; j++) {
            int64_t sl = i * K + j;
            int32_t n0 = m.elem_nodes[a + j], n1 = m.elem_nodes[a + (j + 1) % n];
            double x0 = X(n0), y0 = Y(n0), x1 = X(n1), y1 = Y(n1);
            int32_t eid;
            if (slot_bline[sl] >= 0) {
                int64_t bi = slot_bline[sl];
                int32_t grp = 0;
                for (int64_t g = 0; g + 1 < nGroups; g++)
                    if (bi >= m.b_group_start[g] && bi < m.b_group_start[g + 1]) grp = (int32_t)g;
                if (nGroups > 0 && bi >= m.b_group_start[nGroups - 1]) grp = (int32_t)(nGroups - 1);
                eid = (int32_t)t.e_len.size();
                double dx = x0 - x1, dy = y0 - y1;
                double len = std::sqrt(dx * dx + dy * dy);
                double inv = 1.0 / len;
                t.e_len.push_back(len);
                t.e_nx.push_back(inv * (y1 - y0));
                t.e_ny.push_back(inv * (x0 - x1));
                t.e_mx.push_back(0.5 * (x0 + x1));
                t.e_my.push_back(0.5 * (y0 + y1));
                t.e_node0.push_back(n0);
                t.e_node1.push_back(n1);
                t.e_cell0.push_back((int32_t)i);
                t.e_cell1.push_back(-1);
                t.e_boundary.push_back(1);
                t.e_group.push_back(grp);
                t.g_edge.push_back(eid);
                t.slot_sign[sl] = 1;
            } else if (partner[sl] > sl) {
                eid = (int32_t)t.e_len.size();
                double dx = x0 - x1, dy = y0 - y1;
                double len = std::sqrt(dx * dx + dy * dy);
                double nx = y1 - y0, ny = x0 - x1;
                double mag = std::sqrt(nx * nx + ny * ny);
                t.e_len.push_back(len);
                t.e_nx.push_back(nx / mag);
                t.e_ny.push_back(ny / mag);
                t.e_mx.push_back(0.5 * (x0 + x1));
                t.e_my.push_back(0.5 * (y0 + y1));
                t.e_node0.push_back(n0);
                t.e_node1.push_back(n1);
                t.e_cell0.push_back((int32_t)i);
                t.e_cell1.push_back((int32_t)(partner[sl] / K));
                t.e_boundary.push_back(0);
                t.e_group.push_back(-1);
                t.slot_sign[sl] = 1;
            } else {
                eid = t.slot_edge[partner[sl]];
                t.slot_sign[sl] = -1;
            }
            t.slot_edge[sl] = eid;
            t.perim[i] += t.e_len[eid];
            double det = x0 * y1 - x1 * y0;
            t.area[i] += det;
            t.cx[i] += (x0 + x1) * (x0 * y1 - x1 * y0);
            t.cy[i] += (y0 + y1) * (x0 * y1 - x1 * y0);
        }
        t.area[i] *= 0.5;
        if (!(t.area[i] > 0)) {
            err = "Computed cell " + std::to_string(i) + " area negative";
            return false;
        }
        t.d[i] = (2 * t.area[i]) / t.perim[i];
        t.cx[i] *= 1 / (6 * t.area[i]);
        t.cy[i] *= 1 / (6 * t.area[i]);
    }
    t.E = (int64_t)t.e_len.size();
    t.G = (int64_t)t.g_edge.size();

    // ghost cells: reflected centroid (mesh.d:329-381)
    t.g_cx.resize(t.G);
    t.g_cy.resize(t.G);
    for (int64_t g = 0; g < t.G; g++) {
        int32_t e = t.g_edge[g];
        int32_t o = t.e_cell0[e];
        double nx0 = X(t.e_node0[e]), ny0 = Y(t.e_node0[e]), nx1 = X(t.e_node1[e]), ny1 = Y(t.e_node1[e]);
        double xr, yr;
        if (nx0 != nx1) {
            double x1 = t.cx[o], y1 = t.cy[o];
            double mm = (ny0 - ny1) / (nx0 - nx1);
            double cc = ny0 - mm * nx0;
            double dd = (x1 + (y1 - cc) * mm) / (1.0 + mm * mm);
            xr = 2.0 * dd - x1;
            yr = 2.0 * dd * mm - y1 + 2.0 * cc;
        } else {
            double dd = t.cx[o] - nx0;
            double x1 = t.cx[o];
            xr = -(2.0 * dd - x1);
            yr = t.cy[o];
        }
        t.g_cx[g] = xr;
        t.g_cy[g] = yr;
        t.e_cell1[e] = (int32_t)(C + g);
    }

    // neighbours and least-squares pseudo-inverse gradMat = (A^T A)^-1 A^T (mesh.d:481-642)
    for (int64_t i = 0; i < C; i++) {
        double A[kMaxEdges][2] = {};
        int n = t.nedge[i];
        for (int j = 0; j < n; j++) {
            int32_t e = t.slot_edge[i * K + j];
            int32_t nb = (t.e_cell0[e] == (int32_t)i) ? t.e_cell1[e] : t.e_cell0[e];
            t.slot_nbr[i * K + j] = nb;
            double ncx = nb < C ? t.cx[nb] : t.g_cx[nb - C];
            double ncy = nb < C ? t.cy[nb] : t.g_cy[nb - C];
            A[j][0] = ncx - t.cx[i];
            A[j][1] = ncy - t.cy[i];
        }
        double b[2][2];
        for (int r = 0; r < 2; r++)
            for (int s = 0; s < 2; s++) {
                double acc = 0.0;
                for (int k = 0; k < kMaxEdges; k++) acc += A[k][r] * A[k][s];
                b[r][s] = acc;
            }
        double det = b[0][0] * b[1][1] - b[0][1] * b[1][0];
        double id = 1.0 / det;
        double ci[2][2] = {{b[1][1] * id, -b[0][1] * id}, {-b[1][0] * id, b[0][0] * id}};
        for (int j = 0; j < kMaxEdges; j++) {
            t.gm0[i * K + j] = ci[0][0] * A[j][0] + ci[0][1] * A[j][1];
            t.gm1[i * K + j] = ci[1][0] * A[j][0] + ci[1][1] * A[j][1];
        }
    }
    return true;
}

// Hilbert-curve order of the cell centroids (the curve's index of each centroid on a
// 2^16 x 2^16 grid over the bounding box, by the classic bit-by-bit quadrant
// rotation): consecutive cells form compact patches of the plane, so the cells a
// thread block handles are mostly each other's neighbours.
std::vector<int32_t> hilbert_order(const Topology &t)
{
    const int64_t C = t.C;
    double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
    for (int64_t i = 0; i < C; i++) {
        x0 = std::min(x0, t.cx[i]);
        x1 = std::max(x1, t.cx[i]);
        y0 = std::min(y0, t.cy[i]);
        y1 = std::max(y1, t.cy[i]);
    }
    const double span = std::max(std::max(x1 - x0, y1 - y0), 1e-300);
    const uint32_t n = 1u << 16;
    std::vector<uint64_t> key(C);
    for (int64_t i = 0; i < C; i++) {
        uint32_t x = (uint32_t)std::min<double>(n - 1, std::floor((t.cx[i] - x0) / span * (n - 1)));
        uint32_t y = (uint32_t)std::min<double>(n - 1, std::floor((t.cy[i] - y0) / span * (n - 1)));
        uint64_t d = 0;
        for (uint32_t sq = n / 2; sq > 0; sq /= 2) {
            const uint32_t rx = (x & sq) ? 1 : 0, ry = (y & sq) ? 1 : 0;
            d += (uint64_t)sq * sq * ((3 * rx) ^ ry);
            if (ry == 0) {  // rotate the quadrant
                if (rx == 1) {
                    x = sq - 1 - (x & (sq - 1));
                    y = sq - 1 - (y & (sq - 1));
                }
                std::swap(x, y);
            }
            x &= sq - 1;
            y &= sq - 1;
        }
        key[i] = d;
    }
    std::vector<int32_t> order(C);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
    return order;
}

}  // namespace ebb

using namespace ebb;

extern "C" {

int ebb_mesh_import(const char *path, ebb_mesh **out, char *err, size_t err_len)
{
    if (!path || !out) return EBB_ERR_ARG;
    *out = nullptr;
    std::string p(path);
    // importMesh dispatch (io.d:669-687): gmsh by extension; XFlow/SU2 are not provided
    if (p.find(".msh") == std::string::npos && p.find(".gmsh") == std::string::npos) {
        set_err(err, err_len, "Unsuported mesh format for mesh: " + p);
        return EBB_ERR_FORMAT;
    }
    auto *m = new ebb_mesh();
    std::string e;
    if (!read_gmsh(p, *m, e) || !finish_mesh(*m, e)) {
        delete m;
        set_err(err, err_len, e);
        return e.rfind("cannot open", 0) == 0 ? EBB_ERR_IO : EBB_ERR_FORMAT;
    }
    *out = m;
    return EBB_OK;
}

int ebb_mesh_from_arrays(int64_t n_nodes, const double *xy, int64_t n_elem, const int64_t *elem_off,
                         const int32_t *elem_nodes, int64_t n_b, const int32_t *b_nodes, int32_t n_tags,
                         const int64_t *b_group_start, const char *tags, ebb_mesh **out, char *err, size_t err_len)
{
    if (!out || n_nodes < 0 || n_elem < 0 || n_b < 0 || n_tags < 0 || (n_nodes && !xy) || !elem_off ||
        (n_elem && !elem_nodes) || (n_b && !b_nodes) || (n_tags && (!b_group_start || !tags)))
        return EBB_ERR_ARG;
    auto *m = new ebb_mesh();
    m->xy.assign(xy, xy + 2 * n_nodes);
    m->elem_off.assign(elem_off, elem_off + n_elem + 1);
    int64_t tot = elem_off[n_elem];
    m->elem_nodes.resize(tot);
    for (int64_t i = 0; i < tot; i++) m->elem_nodes[i] = elem_nodes[i] - 1;
    m->b_nodes.assign(b_nodes, b_nodes + 2 * n_b);
    m->b_group_start.assign(b_group_start, b_group_start + n_tags);
    for (int32_t i = 0; i < n_tags; i++) m->tags.emplace_back(tags + (size_t)i * EBB_TAG_LEN);
    std::string e;
    for (int64_t i = 0; i < tot; i++)
        if (m->elem_nodes[i] < 0 || m->elem_nodes[i] >= n_nodes) e = "element references a missing node";
    for (int64_t i = 0; i < 2 * n_b; i++)
        if (m->b_nodes[i] < 0 || m->b_nodes[i] >= n_nodes) e = "line element references a missing node";
    if (e.empty()) finish_mesh(*m, e);
    if (!e.empty()) {
        delete m;
        set_err(err, err_len, e);
        return EBB_ERR_FORMAT;
    }
    *out = m;
    return EBB_OK;
}

int ebb_mesh_get_info(const ebb_mesh *m, ebb_mesh_info *info)
{
    if (!m || !info) return EBB_ERR_ARG;
    std::memset(info, 0, sizeof *info);
    info->n_nodes = (int64_t)m->xy.size() / 2;
    info->n_cells = (int64_t)m->elem_off.size() - 1;
    info->n_tags = (int32_t)m->tags.size();
    info->max_edges = m->max_edges;
    info->face_slots = m->elem_off.back();
    // boundary edges / edges need the topology; count cheaply from the face slots
    std::unordered_map<uint64_t, int> bset;
    for (size_t i = 0; i + 1 < m->b_nodes.size(); i += 2) bset[pair_key(m->b_nodes[i], m->b_nodes[i + 1])] = 1;
    int64_t nb = 0, nonb = 0;
    for (int64_t i = 0; i < info->n_cells; i++) {
        int64_t a = m->elem_off[i];
        int n = (int)(m->elem_off[i + 1] - a);
        for (int j = 0; j < n; j++) {
            if (bset.count(pair_key(m->elem_nodes[a + j], m->elem_nodes[a + (j + 1) % n])))
                nb++;
            else
                nonb++;
        }
    }
    info->n_ghost = nb;
    info->n_int_edges = nonb / 2;
    info->n_edges = nb + nonb / 2;
    return EBB_OK;
}

int ebb_mesh_get_tag(const ebb_mesh *m, int32_t i, char *tag, size_t len)
{
    if (!m || !tag || i < 0 || i >= (int32_t)m->tags.size()) return EBB_ERR_ARG;
    set_err(tag, len, m->tags[i]);
    return EBB_OK;
}

int ebb_mesh_centroids(const ebb_mesh *m, double *xy)
{
    if (!m || !xy) return EBB_ERR_ARG;
    int64_t C = (int64_t)m->elem_off.size() - 1;
    for (int64_t i = 0; i < C; i++) {
        int64_t a = m->elem_off[i];
        int n = (int)(m->elem_off[i + 1] - a);
        double area = 0, cx = 0, cy = 0;
        for (int j = 0; j < n; j++) {
            int32_t n0 = m->elem_nodes[a + j], n1 = m->elem_nodes[a + (j + 1) % n];
            double x0 = m->xy[2 * n0], y0 = m->xy[2 * n0 + 1], x1 = m->xy[2 * n1], y1 = m->xy[2 * n1 + 1];
            area += x0 * y1 - x1 * y0;
            cx += (x0 + x1) * (x0 * y1 - x1 * y0);
            cy += (y0 + y1) * (x0 * y1 - x1 * y0);
        }
        area *= 0.5;
        xy[2 * i] = cx * (1 / (6 * area));
        xy[2 * i + 1] = cy * (1 / (6 * area));
    }
    return EBB_OK;
}

int ebb_mesh_edges(const ebb_mesh *m, int32_t *group, int32_t *cells, double *mid, double *normal, double *len)
{
    if (!m) return EBB_ERR_ARG;
    Topology t;
    std::string e;
    if (!build_topology(*m, t, e)) return EBB_ERR_MESH;
    for (int64_t i = 0; i < t.E; i++) {
        if (group) group[i] = t.e_boundary[i] ? t.e_group[i] : -1;
        if (cells) {
            cells[2 * i] = t.e_cell0[i];
            cells[2 * i + 1] = t.e_cell1[i];
        }
        if (mid) {
            mid[2 * i] = t.e_mx[i];
            mid[2 * i + 1] = t.e_my[i];
        }
        if (normal) {
            normal[2 * i] = t.e_nx[i];
            normal[2 * i + 1] = t.e_ny[i];
        }
        if (len) len[i] = t.e_len[i];
    }
    return EBB_OK;
}

void ebb_mesh_free(ebb_mesh *m) { delete m; }

}  // extern "C"
