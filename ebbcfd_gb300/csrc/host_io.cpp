// host_io.cpp -- .esln v2 solution files (source/io.d:55-161 saveSolution,
// source/io.d:218-366 loadSolution), big-endian.
//
// Layout: u32 magic 0xEA98E1F5, u32 version (2), u32 cells, f64 t, f64 dt, u32 M (4),
// u32 order; per cell in reference order: u32 global id, u8 edge count, 4 f64 state,
// edge count x 4 f64 face states; then 4 CRC-32 bytes.  The reference computes the
// CRC over its whole buffer including the 4 not-yet-written trailing bytes; this
// writer takes those bytes as zero (what a freshly mapped buffer holds).  Readers,
// the reference's included, do not check the CRC.
#include <cstdio>
#include <cstring>
#include <vector>

#include "solver_impl.hpp"

namespace {

uint32_t crc_table[256];
bool crc_init = false;

void init_crc()
{
    for (uint32_t i = 0; i < 256; i++) {
        uint32_t c = i;
        for (int k = 0; k < 8; k++) c = (c & 1) ? (0xEDB88320u ^ (c >> 1)) : (c >> 1);
        crc_table[i] = c;
    }
    crc_init = true;
}

uint32_t crc32(const uint8_t *p, size_t n)
{
    if (!crc_init) init_crc();
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; i++) c = crc_table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

struct BE {
    std::vector<uint8_t> b;
    void u32(uint32_t v)
    {
        for (int k = 3; k >= 0; k--) b.push_back((uint8_t)(v >> (8 * k)));
    }
    void u8(uint8_t v) { b.push_back(v); }
    void f64(double d)
    {
        uint64_t v;
        std::memcpy(&v, &d, 8);
        for (int k = 7; k >= 0; k--) b.push_back((uint8_t)(v >> (8 * k)));
    }
};

// append the CRC-32 (over the body and 4 zero bytes, see above) and write the file
int finish_and_write(BE &w, const char *path)
{
    const size_t body = w.b.size();
    w.b.resize(body + 4, 0);
    uint32_t c = crc32(w.b.data(), w.b.size());
    w.b.resize(body);
    for (int k = 0; k < 4; k++) w.u8((uint8_t)(c >> (8 * k)));
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return EBB_ERR_IO;
    size_t n = std::fwrite(w.b.data(), 1, w.b.size(), fp);
    std::fclose(fp);
    return n == w.b.size() ? EBB_OK : EBB_ERR_IO;
}

struct RD {
    const uint8_t *p, *end;
    bool ok = true;
    uint32_t u32()
    {
        if (end - p < 4) {
            ok = false;
            return 0;
        }
        uint32_t v = ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
        p += 4;
        return v;
    }
    uint8_t u8()
    {
        if (end - p < 1) {
            ok = false;
            return 0;
        }
        return *p++;
    }
    double f64()
    {
        if (end - p < 8) {
            ok = false;
            return 0;
        }
        uint64_t v = 0;
        for (int k = 0; k < 8; k++) v = (v << 8) | p[k];
        p += 8;
        double d;
        std::memcpy(&d, &v, 8);
        return d;
    }
};

}  // namespace

namespace ebb {

// Cells of one .esln file (v1: states in order; v2: global id, edge count, state, face
// states) into q by global id (loadSolution, io.d:218-366, partitioned form).
int read_esln_into(const char *path, std::vector<double> &q, std::vector<uint8_t> &seen, double &t, double &dt)
{
    if (!path) return EBB_ERR_ARG;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return EBB_ERR_IO;
    std::vector<uint8_t> buf;
    uint8_t tmp[1 << 16];
    size_t n;
    while ((n = std::fread(tmp, 1, sizeof tmp, fp)) > 0) buf.insert(buf.end(), tmp, tmp + n);
    std::fclose(fp);
    RD r{buf.data(), buf.data() + buf.size()};
    if (r.u32() != 0xEA98E1F5u || !r.ok) return EBB_ERR_FORMAT;
    const uint32_t ver = r.u32();
    const uint32_t cells = r.u32();
    t = r.f64();
    dt = r.f64();
    const uint64_t C = seen.size();
    if (!r.ok) return EBB_ERR_FORMAT;
    if (ver == 1) {
        if (cells != C) return EBB_ERR_FORMAT;
        for (uint64_t i = 0; i < C; i++) {
            for (int k = 0; k < 4; k++) q[4 * i + k] = r.f64();
            seen[i] = 1;
        }
    } else if (ver == 2) {
        const uint32_t M = r.u32();
        (void)r.u32();
        if (M != 4) return EBB_ERR_FORMAT;
        for (uint32_t c = 0; c < cells && r.ok; c++) {
            const uint32_t id = r.u32();
            const int ne = r.u8();
            if (id >= C) return EBB_ERR_FORMAT;
            for (int k = 0; k < 4; k++) q[4 * (size_t)id + k] = r.f64();
            for (int j = 0; j < ne; j++)
                for (int k = 0; k < 4; k++) (void)r.f64();  // face states are recomputed by the next residual
            seen[id] = 1;
        }
    } else {
        return EBB_ERR_FORMAT;
    }
    return r.ok ? EBB_OK : EBB_ERR_FORMAT;
}

// .esln v2 of points without edges (the refined mesh of ebb-reconstruct,
// reconstruct.d:418-420): entry i = global id i, 0 edges, q[i].
int write_esln_points(const char *path, int64_t n, const double *q, double t, double dt, uint32_t order)
{
    BE w;
    w.b.reserve(40 + (size_t)n * 37);
    w.u32(0xEA98E1F5u);
    w.u32(2);
    w.u32((uint32_t)n);
    w.f64(t);
    w.f64(dt);
    w.u32(4);
    w.u32(order);
    for (int64_t i = 0; i < n; i++) {
        w.u32((uint32_t)i);
        w.u8(0);
        for (int k = 0; k < 4; k++) w.f64(q[4 * i + k]);
    }
    return finish_and_write(w, path);
}

}  // namespace ebb

extern "C" {

int ebb_save_solution(ebb_solver *s, const char *path, double t, double dt)
{
    if (!s || !path) return EBB_ERR_ARG;
    const int64_t C = s->C;
    std::vector<double> q(4 * C), f(4 * s->ref_face_slot.size());
    int r = ebb_get_state(s, q.data());
    if (r) return r;
    if ((r = ebb_get_face_states(s, f.data()))) return r;
    BE w;
    w.b.reserve(40 + C * (5 + 32) + f.size() * 8);
    w.u32(0xEA98E1F5u);
    w.u32(2);
    w.u32((uint32_t)C);
    w.f64(t);
    w.f64(dt);
    w.u32(4);
    w.u32((uint32_t)s->cfg.order);
    size_t fo = 0;
    for (int64_t i = 0; i < C; i++) {
        w.u32((uint32_t)i);
        const int ne = s->ref_nedge[i];
        w.u8((uint8_t)ne);
        for (int k = 0; k < 4; k++) w.f64(q[4 * i + k]);
        for (int j = 0; j < ne; j++, fo++)
            for (int k = 0; k < 4; k++) w.f64(f[4 * fo + k]);
    }
    return finish_and_write(w, path);
}

int ebb_load_solution(ebb_solver *s, const char *path) { return ebb_load_solution_parts(s, 1, &path); }

int ebb_load_solution_parts(ebb_solver *s, int32_t n, const char *const *paths)
{
    if (!s || n <= 0 || !paths) return EBB_ERR_ARG;
    std::vector<double> q(4 * s->C);
    std::vector<uint8_t> seen(s->C, 0);
    double t = 0, dt = 0;
    for (int32_t k = 0; k < n; k++) {
        double tk, dtk;
        int r = ebb::read_esln_into(paths[k], q, seen, tk, dtk);
        if (r) return r;
        if (k == 0) {
            t = tk;
            dt = dtk;
        }
    }
    for (int64_t i = 0; i < s->C; i++)
        if (!seen[i]) return EBB_ERR_FORMAT;  // a cell no file covers
    int rc = ebb_set_state(s, q.data());
    if (rc) return rc;
    return ebb_set_time(s, t, dt);
}

}  // extern "C"
