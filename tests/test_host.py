"""Host side of the C ABI without a GPU: library load and exports, config parsing
(source/config.d:112-313 semantics), gmsh import (source/io.d:689-990 semantics)
checked against the oracle's restatement, and loud failure of the compute entry
points when no device is present."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

import ebbcfd_gb300 as E
from ebbcfd_gb300 import _lib, meshgen
from oracle import gmsh_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "ebb_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ebb_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol():
    L = _lib.load()
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.SIGNATURES, n
    assert L.ebb_abi_version() == 1


def test_struct_layout_matches_binding():
    L = _lib.load()
    a, b, c = C.c_size_t(), C.c_size_t(), C.c_size_t()
    assert L.ebb_struct_sizes(C.byref(a), C.byref(b), C.byref(c)) == 0
    assert a.value == C.sizeof(_lib.Config)
    assert b.value == C.sizeof(_lib.MeshInfo)
    assert c.value == C.sizeof(_lib.StepRecord)


CONFIGS = sorted(f for f in glob.glob(os.path.join(ROOT, "tests", "golden", "meshes", "*.json"))
                 if not f.endswith("manifest.json"))


@pytest.mark.parametrize("path", CONFIGS, ids=[os.path.basename(p) for p in CONFIGS])
def test_config_parse_matches_reference_semantics(path):
    text = open(path).read()
    cfg = E.load_config(text)
    r = gmsh_ref.load_config(text)
    assert cfg.mesh_file.decode() == r["mesh"]
    assert cfg.flux == gmsh_ref.FLUXES[r["flux"]]
    assert cfg.integrator == gmsh_ref.INTEGRATORS[r["integrator"]]
    assert cfg.dt == r["dt"] and cfg.t_end == r["tEnd"] and cfg.cfl == r["CFL"]
    assert cfg.save_iter == r["saveIter"] and cfg.plot_iter == r["plotIter"]
    assert bool(cfg.limited) == r["limited"] and bool(cfg.dynamic_dt) == r["dynamicDt"]
    assert bool(cfg.local_timestep) == r["localTimestep"] and bool(cfg.viscosity) == r["viscosity"]
    assert bool(cfg.cfl_adjust) == r["cflAdjust"] and bool(cfg.multistage_limiting) == r["multistageLimiting"]
    assert cfg.lp_thresh == r["lpThresh"] and cfg.order == r["order"]
    assert list(cfg.ic) == r["ic"]
    pc = r["physicalConfig"]
    assert (cfg.pr, cfg.r_gas, cfg.re, cfg.l_ref) == (pc["Pr"], pc["R"], pc["Re"], pc["L"])
    assert cfg.n_boundaries == len(r["boundaries"])
    for i, b in enumerate(r["boundaries"]):
        B = cfg.boundaries[i]
        assert B.tag.decode() == b["tag"] and B.type == b["type"]
        assert [B.data[k] for k in range(B.n_data)] == b["q"]
    assert [cfg.force_boundary[k].value.decode() for k in range(cfg.n_force)] == r["forceBoundary"]


BASE = """{"mesh": "m.msh", "dt": 0.001, "tEnd": 1, "flux": "roeFlux", "saveIter": -1, "plotIter": -1,
 "forceBoundary": ["Wall", "Other"], "initialConditions": [0.5, 0, 1, 1],
 "boudaryConditions": [{"tag": "Wall", "type": "madeUpType", "q": [0.5, 0, 1, 1]}] %s}"""


def test_config_defaults_and_quirks():
    c = E.load_config(BASE % "")
    # absent keys take the reference defaults (config.d:137-260)
    assert c.cfl == 0.5 and c.dynamic_dt == 1 and c.integrator == 0 and c.limited == 1
    assert c.local_timestep == 0 and c.lp_thresh == -1 and c.order == 2 and c.multistage_limiting == 1
    assert c.cfl_adjust == 1 and c.viscosity == 0 and (c.pr, c.r_gas, c.re, c.l_ref) == (0.7, 8.3145, 1000, 1)
    # unknown boundary type keeps the enum default FullState (config.d:273-301)
    assert c.boundaries[0].type == 0
    assert c.n_force == 2
    # present flags are true only when JSON true
    c = E.load_config(BASE % ', "limited": 1, "dynamicDt": false, "order": 3, "CFL": 2')
    assert c.limited == 0 and c.dynamic_dt == 0 and c.order == 2 and c.cfl == 2.0
    # a partial physicalConfig falls back to all defaults
    c = E.load_config(BASE % ', "physicalConfig": {"Pr": 0.9}')
    assert c.pr == 0.7
    # dt must be a floating-point literal (config.d:119 uses .floating)
    with pytest.raises(E.EbbError):
        E.load_config((BASE % "").replace('"dt": 0.001', '"dt": 1'))
    with pytest.raises(E.EbbError):
        E.load_config((BASE % "").replace('"roeFlux"', '"hllFlux"'))
    with pytest.raises(E.EbbError):
        E.load_config("{not json")
    # single-string forceBoundary
    c = E.load_config((BASE % "").replace('["Wall", "Other"]', '"Wall"'))
    assert c.n_force == 1 and c.force_boundary[0].value == b"Wall"


MESHES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "meshes", "*.msh")))


@pytest.mark.parametrize("path", MESHES, ids=[os.path.basename(p) for p in MESHES])
def test_gmsh_import_matches_reference_reader(path):
    m = E.import_mesh(path)
    r = gmsh_ref.parse_gmsh(path)
    assert m.n_cells == len(r["elements"])
    assert m.tags == r["bTags"]
    assert m.info.face_slots == sum(len(e) for e in r["elements"])
    # centroids follow the CCW-corrected element orientation
    xy = m.centroids()
    for i in (0, len(xy) // 2, len(xy) - 1):
        el = np.array(r["elements"][i]) - 1
        p = r["nodes"][el]
        assert np.allclose(xy[i], p.mean(axis=0), atol=0.5 * np.ptp(p, axis=0).max())


@pytest.mark.parametrize("path", MESHES[:4], ids=[os.path.basename(p) for p in MESHES[:4]])
def test_mesh_edges_match_the_oracle_edges(path):
    """ebb_mesh_edges lists the reference's edges (mesh.d:242-313 creation order) with
    the oracle's lengths, normals, midpoints and cell indices, and the boundary group
    of each boundary edge."""
    from oracle import ref
    r = gmsh_ref.parse_gmsh(path)
    conf = {"dt": 1e-4, "dynamicDt": True, "tEnd": 1.0, "flux": "roeFlux", "integrator": "Euler", "limited": True,
            "lpThresh": -1, "order": 2, "CFL": 0.5, "ic": [0.5, 0, 1, 1], "localTimestep": False,
            "multistageLimiting": True, "cflAdjust": False, "viscosity": False,
            "physicalConfig": {"Pr": 0.7, "R": 8.3145, "Re": 1000, "L": 1},
            "boundaries": [{"tag": t, "type": 0, "q": [0.5, 0, 1, 1]} for t in r["bTags"]], "forceBoundary": []}
    om = ref.OracleMesh(r, conf)
    eg = om.geometry()["edge"]
    e = E.import_mesh(path).edges()
    assert len(e["len"]) == om.n_edges
    assert np.array_equal(e["len"], eg[:, 0]) and np.array_equal(e["normal"], eg[:, 1:3])
    assert np.array_equal(e["mid"], eg[:, 3:5]) and np.array_equal(e["cells"], eg[:, 5:7].astype(np.int32))
    assert np.array_equal(e["group"] >= 0, eg[:, 7] != 0)
    assert set(e["group"][e["group"] >= 0]) <= set(range(len(r["bTags"])))


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


SPLIT = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
3
1 1 "Bottom"
1 2 "Rest"
2 3 "Flow"
$EndPhysicalNames
$Nodes
4
1 0 0 0
2 1 0 0
3 1 1 0
4 0 1 0
$EndNodes
$Elements
6
1 1 2 1 1 1 2
2 1 2 2 2 2 3
3 1 2 2 2 3 4
4 1 2 1 1 4 1
5 2 2 3 3 1 3 2
6 2 2 3 3 1 3 4
$EndElements
"""


def test_gmsh_split_groups_and_clockwise_elements(tmp_path):
    """Group 'Bottom' appears twice (merged, io.d:910-942); element 5 is clockwise (reversed, io.d:969-987)."""
    p = write(tmp_path, "split.msh", SPLIT)
    r = gmsh_ref.parse_gmsh(p)
    assert r["bTags"] == ["Bottom", "Rest"]
    assert r["bGroupStart"] == [0, 2]
    assert [list(x) for x in r["bNodes"]] == [[0, 1], [3, 0], [1, 2], [2, 3]]
    assert r["elements"][0] == [2, 3, 1]
    m = E.import_mesh(p)
    assert m.n_cells == 2 and m.tags == ["Bottom", "Rest"] and m.info.n_ghost == 4
    assert m.info.n_int_edges == 1


@pytest.mark.parametrize("bad,needle", [
    ("$MeshFormat\n2.2 1 8\n$EndMeshFormat\n", "format"),
    (SPLIT.replace("1 2 2 2 2 3", "9 2 2 2 2 3"), "element"),
    (SPLIT.replace("5 2 2 3 3 1 3 2", "5 15 2 3 3 1"), "type"),
    (SPLIT.replace("3 1 1 0", "3 1 1"), "node"),
    (SPLIT.replace("$EndNodes", "$EndNodez").replace("$Elements", "$Junk"), ""),
])
def test_gmsh_malformed_inputs_fail_cleanly(tmp_path, bad, needle):
    p = write(tmp_path, "bad.msh", bad)
    with pytest.raises(E.EbbError) as ei:
        E.import_mesh(p)
    assert ei.value.code in (3, 4)


def test_missing_mesh_file_is_io_error():
    with pytest.raises(E.EbbError) as ei:
        E.import_mesh("/nonexistent/none.msh")
    assert ei.value.code == 2


def test_mesh_from_arrays_and_generators():
    g = meshgen.wedge(3000, seed=0)
    m = g.to_solver_mesh()
    assert m.n_cells == g.n_cells
    assert m.tags == g.tags
    assert m.info.n_ghost == len(g.b_nodes)
    q = meshgen.uniform_quads(8).to_solver_mesh()
    assert q.n_cells == 64 and q.info.n_ghost == 32 and q.info.n_int_edges == 112
    f = meshgen.flat_plate(20000)
    fm = f.to_solver_mesh()
    assert fm.n_cells == f.n_cells and fm.info.max_edges == 4


def test_solver_create_fails_loudly_without_gpu():
    L = _lib.load()
    n = C.c_int()
    if L.ebb_device_count(C.byref(n)) == 0:
        pytest.skip("a GPU is present; the no-device path is not reachable")
    m = meshgen.uniform_quads(4).to_solver_mesh()
    cfg = E.default_config()
    E.set_boundaries(cfg, [("Freestream", "fullState", [0.5, 0, 1, 1])])
    with pytest.raises(E.EbbError) as ei:
        E.UfvmSolver(m, cfg)
    assert ei.value.code == 10
    with pytest.raises(E.EbbError):
        E.roe_flux(np.ones(4), np.ones(4), [1.0, 0.0])


@pytest.mark.parametrize("cname,pyname", [("ebb_instance_status", "InstanceStatus"),
                                           ("ebb_server_options", "ServerOptions"),
                                           ("ebb_request_result", "RequestResult"),
                                           ("ebb_server_stats", "ServerStats")])
def test_struct_layout_matches_header(tmp_path, cname, pyname):
    """Field offsets and size of a public struct as a C compiler lays it out from the
    header vs the ctypes binding."""
    import subprocess
    st = getattr(_lib, pyname)
    names = [f[0] for f in st._fields_]
    body = "".join('printf("%%zu ", offsetof(%s, %s));' % (cname, n) for n in names)
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "ebb_gb300.h"\nint main(void){%s'
                   'printf("%%zu\\n", sizeof(%s));return 0;}\n' % (body, cname))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [getattr(st, n).offset for n in names] + [C.sizeof(st)]
    assert got == want


def _bump(n, mach=0.5, seed=0, **kw):
    m = meshgen.bump_channel(n, h=0.05, seed=seed).to_solver_mesh()
    cfg = E.default_config()
    q = [mach, 0, 1, 1]
    E.set_boundaries(cfg, [("Inflow", "fullState", q), ("Outflow", "fullState", q), ("Wall", "inviscidWall", q)])
    for k, v in kw.items():
        setattr(cfg, k, v)
    return m, cfg


def test_batch_footprint_without_device():
    a = _bump(1500, seed=1)
    b = _bump(4000, mach=0.7, seed=2)
    fa = E.batch_footprint([a[0]], [a[1]])
    fb = E.batch_footprint([b[0]], [b[1]])
    fab = E.batch_footprint([a[0], b[0]], [a[1], b[1]])
    assert fa > 1500 * 500 and fb > fa
    assert 0.9 * (fa + fb) < fab < 1.1 * (fa + fb)
    assert E.batch_footprint([a[0]], [a[1]], "split") < fa
    # per-cell bytes are flat in the mesh size
    assert abs(fa / a[0].n_cells - fb / b[0].n_cells) < 0.25 * fa / a[0].n_cells
    bad = E.default_config()
    with pytest.raises(E.EbbError) as ei:
        E.batch_footprint([a[0]], [bad])
    assert ei.value.code == 5


def test_batch_create_fails_loudly_without_gpu():
    L = _lib.load()
    n = C.c_int()
    if L.ebb_device_count(C.byref(n)) == 0:
        pytest.skip("a GPU is present; the no-device path is not reachable")
    a = _bump(800)
    with pytest.raises(E.EbbError) as ei:
        E.UfvmBatch([a[0], a[0]], [a[1], a[1]])
    assert ei.value.code == 10


def test_server_create_fails_loudly_without_gpu():
    L = _lib.load()
    n = C.c_int()
    if L.ebb_device_count(C.byref(n)) == 0:
        pytest.skip("a GPU is present; the no-device path is not reachable")
    with pytest.raises(E.EbbError) as ei:
        E.EbbServer("split")
    assert ei.value.code == 10


def test_server_option_defaults():
    """ebb_server_options_defaults (no device needed): split requests, finishing of
    stalled split solves on, in plain FP64, after 1000 stalled iterations; the Python
    mirror maps precision names for the finishing form."""
    L = _lib.load()
    o = _lib.ServerOptions()
    L.ebb_server_options_defaults(C.byref(o))
    from ebbcfd_gb300.solver import PRECISION
    assert o.precision == PRECISION["split"] == 1
    assert o.finish_fp64 == 1 and o.stall_steps == 1000 and o.finish_precision == PRECISION["fp64"] == 0
    assert o.escalate == 0 and o.max_batch == 512 and o.hbm_budget == 150_000_000_000
    assert PRECISION["df"] == 2


def test_cylinder_generator():
    g = meshgen.cylinder(5000, seed=3)
    m = g.to_solver_mesh()
    assert 0.8 * 5000 < m.n_cells < 1.25 * 5000
    assert m.tags == ["Inflow", "Outflow", "Top", "Bottom", "Cylinder"]
    xy = m.centroids()
    assert (np.hypot(xy[:, 0], xy[:, 1]) > 0.5).all()
    assert xy[:, 0].min() > -10 and xy[:, 0].max() < 30 and np.abs(xy[:, 1]).max() < 10


def test_bump_channel_mesh_follows_the_bump():
    """No triangle of the channel lies under the bump (the Delaunay hull covers that
    region) and the Poisson-disk points leave no poorly shaped triangle (quality
    4 sqrt(3) area / sum of squared edges, 1 for equilateral, above 0.3)."""
    h = 0.1
    g = meshgen.bump_channel(6000, h=h, seed=212)
    tr = np.asarray(g.elements) - 1
    p = g.nodes[tr]
    c = p.mean(axis=1)
    floor = np.where((c[:, 0] >= 1) & (c[:, 0] <= 2), h * np.sin(np.pi * (c[:, 0] - 1)) ** 2, 0.0)
    assert (c[:, 1] > floor).all()
    a = 0.5 * ((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    l2 = ((p[:, 1] - p[:, 0]) ** 2).sum(1) + ((p[:, 2] - p[:, 1]) ** 2).sum(1) + ((p[:, 0] - p[:, 2]) ** 2).sum(1)
    assert (4 * np.sqrt(3) * a / l2).min() > 0.3


BITCONV_CHECK = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "bitconv.h"
static uint32_t fb(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
static uint64_t db(double x) { uint64_t u; std::memcpy(&u, &x, 8); return u; }
static float bf(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }
static double bd(uint64_t u) { double x; std::memcpy(&x, &u, 8); return x; }
static long bad = 0, n = 0;
static void check_d2f(uint64_t u) {
    double d = bd(u);
    uint32_t got = ebbbits::d2f_bits((uint32_t)(u >> 32), (uint32_t)u);
    n++;
    if (std::isnan(d)) { if (!std::isnan(bf(got))) bad++; return; }
    uint32_t want = std::fabs(d) < 0x1p-126 ? (uint32_t)(u >> 32) & 0x80000000u : fb((float)d);
    if (got != want) { if (bad < 5) std::printf("d2f %016llx got %08x want %08x\n", (unsigned long long)u, got, want); bad++; }
}
static void check_f2d(uint32_t f) {
    float x = bf(f);
    uint64_t got = ebbbits::f2d_bits(f);
    n++;
    if (std::isnan(x)) { if (!std::isnan(bd(got))) bad++; return; }
    uint64_t want = ((f >> 23) & 0xffu) == 0 ? (uint64_t)(f & 0x80000000u) << 32 : db((double)x);
    if (got != want) { if (bad < 5) std::printf("f2d %08x got %016llx\n", f, (unsigned long long)got); bad++; }
}
int main() {
    std::mt19937_64 rng(7);
    for (uint64_t f = 0; f < (1ull << 32); f += 9973) check_f2d((uint32_t)f);
    const uint32_t fe[] = {0u, 0x80000000u, 1u, 0x807fffffu, 0x00800000u, 0x7f7fffffu, 0xff7fffffu,
                           0x7f800000u, 0xff800000u, 0x7fc00000u, 0x7f800001u, 0x3f800000u, 0xbf800001u};
    for (uint32_t f : fe) check_f2d(f);
    for (int k = 0; k < 4000000; k++) check_d2f(rng());
    for (int k = 0; k < 4000000; k++) {  // doubles in and near the FP32 range, ties included
        uint64_t e = 896 + rng() % 260, m = rng() & 0xfffffffffffffull;
        if (k & 1) m = (m & ~0x1fffffffull) | 0x10000000ull;
        if (k % 3 == 0) m |= 0x1fffffffull;
        check_d2f(((rng() & 1) << 63) | (e << 52) | m);
    }
    const double de[] = {0.0, -0.0, 1.0, -1.0, 0x1p-126, 0x1p-127, -0x1.fffffffp-127, 0x1.fffffep127,
                         0x1.ffffffp127, 0x1.fffffefffffffp127, 3.4028235677973366e38, INFINITY, -INFINITY,
                         NAN, 1e-300, 1e300, 0.1, 1.0 / 3.0};
    for (double d : de) check_d2f(db(d));
    // truncating conversion for range filters: below 2^-23 relative in [2^-126, 2^128),
    // never larger in magnitude than the double, signed zero below, signed infinity above
    for (int k = 0; k < 4000000; k++) {
        uint64_t u = k < 2000000 ? rng() : (((rng() & 1) << 63) | ((uint64_t)(880 + rng() % 290) << 52) |
                                            (rng() & 0xfffffffffffffull));
        double d = bd(u);
        float f = bf(ebbbits::d2f_trunc_bits((uint32_t)(u >> 32), (uint32_t)u));
        n++;
        double a = std::fabs(d);
        bool ok;
        if (std::isnan(d) || a >= 0x1p128) ok = std::isinf(f) && std::signbit(f) == std::signbit(d);
        else if (a < 0x1p-126) ok = f == 0.0f && std::signbit(f) == std::signbit(d);
        else ok = std::fabs((double)f) <= a && (a - std::fabs((double)f)) < 0x1p-23 * a &&
                  std::signbit(f) == std::signbit(d);
        if (!ok) { if (bad < 5) std::printf("trunc %016llx -> %a\n", (unsigned long long)u, f); bad++; }
    }
    std::printf("%ld %ld\n", n, bad);
    return 0;
}
"""


def test_integer_pipe_conversions_match_ieee(tmp_path):
    """The split path's integer-pipe float<->double conversions (csrc/bitconv.h) give
    the host's IEEE conversions bit for bit: every 9973rd FP32 pattern, 8M doubles
    (random patterns and values in and near the FP32 range with exact ties), and the
    edge values; subnormal FP32 results and inputs become signed zeros.  The truncating
    conversion of the FP64 kernels' range filters stays within 2^-23 below the value
    (signed zero under FP32's normal range, signed infinity above it) on 4M doubles."""
    import subprocess
    src = tmp_path / "bitconv_check.cpp"
    src.write_text(BITCONV_CHECK)
    exe = tmp_path / "bitconv_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "ebbcfd_gb300", "csrc"), str(src),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    n, bad = int(out[-2]), int(out[-1])
    assert n > 12_000_000 and bad == 0, " ".join(out[:-2])


DFLOAT_CHECK = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "dfloat.h"
using ebbdf::df;
typedef long double L;
static L val(df a) { return (L)a.hi + (L)a.lo; }
static std::mt19937_64 rng(11);
static double u01() { return (rng() >> 11) * 0x1p-53; }
static df rnd(int emax) {
    double m = 1.0 + u01();
    int e = (int)(rng() % (2 * emax + 1)) - emax;
    double x = std::ldexp(m, e) * ((rng() & 1) ? -1.0 : 1.0);
    return df(x);
}
int main() {
    const double U = 0x1p-46;
    double emul = 0, ediv = 0, esqrt = 0, eadd = 0, eaddc = 0, econv = 0, emulf = 0, echain = 0, edot = 0;
    long n = 0;
    for (int k = 0; k < 2000000; k++) {
        df a = rnd(20), b = rnd(20);
        L va = val(a), vb = val(b);
        L r;
        r = va * vb; emul = std::fmax(emul, (double)(std::fabs(val(a * b) - r) / std::fabs(r)) / U);
        r = va / vb; ediv = std::fmax(ediv, (double)(std::fabs(val(a / b) - r) / std::fabs(r)) / U);
        float f = b.hi;
        r = va * (L)f; emulf = std::fmax(emulf, (double)(std::fabs(val(ebbdf::mul_f(a, f)) - r) / std::fabs(r)) / U);
        df pa = ebbdf::fabs(a);
        r = std::sqrt(val(pa)); esqrt = std::fmax(esqrt, (double)(std::fabs(val(ebbdf::sqrt(pa)) - r) / r) / U);
        r = va + vb; eadd = std::fmax(eadd, (double)(std::fabs(val(a + b) - r) / (std::fabs(va) + std::fabs(vb))) / U);
        // cancellation: b close to -a
        df c = -(a * df(1.0 + std::ldexp(u01(), -(int)(rng() % 40))));
        L vc = val(c);
        r = va + vc; eaddc = std::fmax(eaddc, (double)(std::fabs(val(a + c) - r) / (std::fabs(va) + std::fabs(vc))) / U);
        // chains: a product of products, and a sum of two products (relative to the
        // summed magnitudes)
        df e = rnd(10);
        L ve = val(e);
        r = va * vb * ve;
        echain = std::fmax(echain, (double)(std::fabs(val((a * b) * e) - r) / std::fabs(r)) / U);
        r = va * vb + vc * ve;
        edot = std::fmax(edot, (double)(std::fabs(val(a * b + c * e) - r) / (std::fabs(va * vb) + std::fabs(vc * ve))) / U);
        double x = std::ldexp(1.0 + u01(), (int)(rng() % 121) - 60) * ((rng() & 1) ? -1.0 : 1.0);
        econv = std::fmax(econv, (double)(std::fabs(val(df(x)) - (L)x) / std::fabs((L)x)) / U);
        n++;
    }
    std::printf("%ld %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f %.3f\n", n, emul, emulf, ediv, esqrt, eadd, eaddc, econv,
                echain, edot);
}
"""


def test_double_float_error_bounds(tmp_path):
    """The double-float arithmetic of the df precision form (csrc/dfloat.h) against
    80-bit (x86) or 128-bit (Arm) long double references on 2M random operand pairs
    over 2^+-20 of both signs: product, product by an FP32 number, quotient and square
    root within 2 units of 2^-46 of the exact result (relative); sums within 2 units of
    2^-46 of |a| + |b|, with near-cancelling pairs as well; the conversion from double
    within 2^-48; a product of products and a sum of two products (their operands not
    renormalised) within 4 units of 2^-46 (relative to the summed magnitudes)."""
    import subprocess
    src = tmp_path / "dfcheck.cpp"
    src.write_text(DFLOAT_CHECK)
    exe = tmp_path / "dfcheck"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "ebbcfd_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    n = int(out[0])
    emul, emulf, ediv, esqrt, eadd, eaddc, econv, echain, edot = (float(x) for x in out[1:])
    assert n == 2_000_000
    assert max(emul, emulf, ediv, esqrt, eadd, eaddc) <= 2.0, out
    assert econv <= 0.25, out
    assert max(echain, edot) <= 4.0, out


def test_hanging_node_polygons():
    """The non-conforming quad mesh used by the six-neighbour parity case: 14 pentagons
    and one hexagon among the quads, counter-clockwise and tiling the unit square; the
    product's mesh import and the oracle's restatement agree on cells and edges."""
    from oracle import ref
    from tests.cases import cfg_json
    g = meshgen.hanging_quads(16)
    els = g.element_list()
    sizes = np.bincount([len(e) for e in els])
    assert sizes[4] == 817 and sizes[5] == 14 and sizes[6] == 1
    area = 0.0
    for e in els:
        p = g.nodes[np.asarray(e) - 1]
        a = 0.5 * np.sum(p[:, 0] * np.roll(p[:, 1], -1) - np.roll(p[:, 0], -1) * p[:, 1])
        assert a > 0
        area += a
    assert abs(area - 1.0) < 1e-12
    m = g.to_solver_mesh()
    assert m.info.max_edges == 6 and m.n_cells == len(els)
    text = cfg_json(initialConditions=[0.5, 0, 1, 1],
                    boudaryConditions=[{"tag": "Freestream", "type": "dirichlet", "q": [0.5, 0, 1, 1]}])
    om = ref.OracleMesh(g.as_reader_dict(), gmsh_ref.load_config(text), mms=2)
    assert om.n_cells == m.n_cells and om.n_bnd == len(g.b_nodes)
    assert om.n_int == m.info.n_int_edges


def test_bench_roofline_inputs():
    """bench.py's roofline inputs: the committed ncu summaries carry DRAM traffic for
    every stage kernel of both precision forms on the wedge and of all three on the
    plate (scaled by cell count), the FP64 kernels' FP64-pipe share and the
    double-float kernels' FMA-pipe share, and the algorithmic-bytes model counts the
    split update's freestream-correction reads and the viscous gradient traffic."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    wl, cells = bench.WEDGE_WORKLOAD, 1001045
    for kern in ("k_cell", "k_flux", "k_update"):
        for prec in ("fp64", "split"):
            t = bench.profiled_counters(kern, prec, wl, cells)["traffic"]
            assert t is not None and t["bytes"] > 1e7 and t["captured_cells"] == cells, (kern, prec)
            half = bench.profiled_counters(kern, prec, wl, cells // 2)["traffic"]
            assert abs(half["bytes"] - t["bytes"] * (cells // 2) / cells) <= 1.0
        assert bench.profiled_counters(kern, "fp64", wl, cells)["fp64_pipe_pct"] > 50
    assert bench.profiled_counters("k_flux", "fp64", "no-such-workload", cells)["traffic"] is None
    # the headline plate: every kernel of the three forms, and the double-float kernels'
    # FMA-pipe share
    for kern in ("k_cell", "k_flux", "k_update"):
        for prec in ("fp64", "split", "df"):
            t = bench.profiled_counters(kern, prec, bench.PLATE_WORKLOAD, 1001778)["traffic"]
            assert t is not None and t["bytes"] > 1e8 and t["captured_cells"] == 1001778, (kern, prec)
        assert bench.profiled_counters(kern, "df", bench.PLATE_WORKLOAD, 1001778)["fma_pipe_pct"] > 10

    class Info:
        n_cells, face_slots, n_int_edges, n_ghost = 1000, 3000, 1480, 40
    b64 = bench.algorithmic_bytes(Info, real=8)
    b32 = bench.algorithmic_bytes(Info, real=4)
    assert all(v > 0 for v in b64.values()) and b32["cell"] < b64["cell"]
    plain32 = Info.n_cells * (4 + 12 + 32 + 16 + 16) + Info.face_slots * 4 + (Info.n_int_edges + Info.n_ghost) * 20
    assert b32["update"] == plain32 + Info.n_cells * 16 + Info.face_slots * 12
    v64 = bench.algorithmic_bytes(Info, real=8, need_grad=True)
    assert v64["flux"] == b64["flux"] + Info.n_int_edges * 8 + (Info.n_cells + Info.n_ghost) * 64
    assert v64["cell"] == b64["cell"] + Info.n_cells * 64


def test_bench_wall_skin_friction():
    """Cf per wall edge from the edge fluxes: 2 * (len F1) / len on the tagged edges,
    sorted by x; other edges are ignored."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    edges = {"group": np.array([-1, 2, 2, 0]), "mid": np.array([[0.5, 0.1], [0.7, 0.0], [0.2, 0.0], [0.1, 0.5]]),
             "len": np.array([1.0, 0.5, 0.25, 1.0])}
    efl = np.array([[0, 9, 0, 0], [0, 0.01, 0, 0], [0, 0.005, 0, 0], [0, 7, 0, 0]], dtype=float)
    x, cf = bench.wall_cf(edges, efl, 2)
    assert np.array_equal(x, [0.2, 0.7]) and np.allclose(cf, [0.04, 0.04])


def test_wedge_mesh_quality_and_count():
    """The benchmark wedge generator: Poisson-disk points give no poorly shaped
    triangle (quality 4 sqrt(3) area / sum of squared edges above 0.35), the triangle
    count lands within 2% of the request, and every boundary edge lies on the domain
    outline with the tag of its segment."""
    n = 20000
    g = meshgen.wedge(n, seed=0)
    tr = np.asarray(g.elements) - 1
    p = g.nodes[tr]
    a = 0.5 * ((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    l2 = ((p[:, 1] - p[:, 0]) ** 2).sum(1) + ((p[:, 2] - p[:, 1]) ** 2).sum(1) + ((p[:, 0] - p[:, 2]) ** 2).sum(1)
    assert (a > 0).all() and (4 * np.sqrt(3) * a / l2).min() > 0.35
    assert abs(len(tr) / n - 1) < 0.02
    ta = np.tan(np.radians(15.0))
    starts = list(g.b_group_start) + [len(g.b_nodes)]
    for t, tag in enumerate(g.tags):
        mid = g.nodes[g.b_nodes[starts[t]:starts[t + 1]]].mean(axis=1)
        x, y = mid[:, 0], mid[:, 1]
        if tag == "Inflow":
            assert np.allclose(x, 0)
        elif tag == "Outflow":
            assert np.allclose(x, 3)
        elif tag == "Top":
            assert np.allclose(y, 1)
        elif tag == "Symmetry":
            assert np.allclose(y, 0) and (x <= 0.5 + 1e-12).all()
        elif tag == "Ramp":
            assert np.allclose(y, (x - 0.5) * ta) and (x >= 0.5 - 1e-12).all()


FDIV_CHECK = r"""
#include <cstdio>
#include <cstdlib>
#include <random>
#include "fdiv.h"
static double fromb(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
int main(int argc, char **argv) {
    long N = atol(argv[1]);
    std::mt19937_64 rng(777);
    long n = 0, bad = 0, fast = 0;
    for (long i = 0; i < N; i++) {
        uint64_t mb = rng() & 0xfffffffffffffull, ma = rng() & 0xfffffffffffffull;
        int eb = (int)(rng() % 261) - 130, ea = (int)(rng() % 621) - 310;
        if (i % 7 == 0) mb &= ~((1ull << (rng() % 52)) - 1);
        if (i % 13 == 0) mb = 0xfffffffffffffull - (rng() % 64);
        if (i % 17 == 0) mb = rng() % 64;
        double b = fromb(((uint64_t)(eb + 1023) << 52) | mb) * ((rng() & 1) ? -1 : 1);
        double a = fromb(((uint64_t)(ea + 1023) << 52) | ma) * ((rng() & 1) ? -1 : 1);
        if (i % 19 == 0) a = (rng() & 1) ? 0.0 : -0.0;
        if (i % 23 == 0) a = b * fromb(((uint64_t)(1023 + (int)(rng() % 9) - 4) << 52) | (rng() % 4096));
        ebbdiv::Recip R = ebbdiv::recip(b);
        double q = ebbdiv::div(a, R), want = a / b;
        n++;
        fast += R.ok;
        if (ebbdiv::bits_of(q) != ebbdiv::bits_of(want)) {
            if (bad < 5) printf("mismatch %a / %a: %a, want %a\n", a, b, q, want);
            bad++;
        }
    }
    printf("%ld %ld %ld\n", n, fast, bad);
    return 0;
}
"""


def test_shared_reciprocal_division_is_ieee(tmp_path):
    """csrc/fdiv.h (one correctly rounded reciprocal shared by several quotients,
    Markstein's correction per quotient) gives the IEEE double quotient bit for bit:
    4M random numerators and divisors over wide exponent ranges, significands near
    all ones and near powers of two, signed zeros and exact quotients.  (300M such
    quotients were checked the same way when it was written, and 1e9 with the seed's
    conversions on bit patterns.)"""
    import subprocess
    src = tmp_path / "fdiv_check.cpp"
    src.write_text(FDIV_CHECK)
    exe = tmp_path / "fdiv_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "ebbcfd_gb300", "csrc"), str(src),
                    "-o", str(exe)], check=True)
    n, fast, bad = (int(x) for x in subprocess.run([str(exe), "4000000"], capture_output=True, text=True,
                                                   check=True).stdout.split()[-3:])
    assert n == 4000000 and fast > 0.9 * n and bad == 0


def _c_struct_fields(text, name):
    """Field names, in order, of `typedef struct [tag] { ... } name;` in C source."""
    import re
    m = re.search(r"typedef struct(?: \w+)? \{([^}]*)\} " + name + r";", text)
    return _field_names(m.group(1))


def _d_struct_fields(text, name):
    import re
    m = re.search(r"struct " + name + r"\s*\{([^}]*)\}", text)
    return _field_names(m.group(1))


def _field_names(body):
    import re
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    body = re.sub(r"//[^\n]*", "", body)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r"\[[^\]]*\]", "", decl)  # array extents (C after the name, D after the type)
        parts = [p.strip() for p in decl.split(",")]
        names.append(parts[0].split()[-1])
        names.extend(p.split()[-1] for p in parts[1:])
    return names


def test_d_binding_mirrors_the_header():
    """ebbcfd_gb300/d/ebb/gb300.d (the D host's extern(C) binding) declares every
    function of include/ebb_gb300.h with the same number of parameters, and every
    public struct with the header's fields in the header's order."""
    import re
    hdr = open(os.path.join(ROOT, "include", "ebb_gb300.h")).read()
    dsrc = open(os.path.join(ROOT, "ebbcfd_gb300", "d", "ebb", "gb300.d")).read()
    h = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    d = re.sub(r"//[^\n]*", "", re.sub(r"/\+.*?\+/", "", dsrc, flags=re.S))

    def protos(text):
        out = {}
        for m in re.finditer(r"\b(?:int|void)\s+(ebb_\w+)\s*\(([^;]*?)\)\s*;", text, flags=re.S):
            args = m.group(2).strip()
            out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
        return out

    ph, pd = protos(h), protos(d)
    assert len(ph) >= 50 and ph == pd, set(ph.items()) ^ set(pd.items())
    for name in ("ebb_config", "ebb_boundary", "ebb_mesh_info", "ebb_step_record", "ebb_instance_status",
                 "ebb_server_options", "ebb_request_result", "ebb_server_stats"):
        assert _c_struct_fields(hdr, name) == _d_struct_fields(dsrc, name), name


def test_esln_fixture_was_read_by_the_reference_reader():
    """tests/golden/esln: the solution file the library wrote for a parity case, with
    what the reference's reader (EbbUtils.importEbbSolution) found in it when the
    fixture was made: version 2, M = 4, and cell averages, global ids, edge counts and
    edge values equal to the oracle's."""
    import hashlib
    import json
    d = os.path.join(ROOT, "tests", "golden", "esln")
    chk = json.load(open(os.path.join(d, "reader_check.json")))
    assert hashlib.sha256(open(os.path.join(d, chk["file"]), "rb").read()).hexdigest() == chk["sha256"]
    f = chk["found"]
    assert f["version"] == 2 and f["M"] == 4 and f["n_cells"] > 100
    assert all(f[k] for k in ("cell_averages_equal_oracle_state", "global_ids_in_cell_order",
                              "edge_counts_equal_elements", "edge_values_equal_oracle_face_states"))
