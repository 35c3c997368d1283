"""ctypes front end of the C oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from . import gmsh_ref

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.c")
LIB = os.path.join(HERE, "_build", "liboracle.so")

MAX_BC = 32


class OCfg(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("dynamicDt", C.c_int),
        ("tEnd", C.c_double),
        ("flux", C.c_int),
        ("integrator", C.c_int),
        ("limited", C.c_int),
        ("lpThresh", C.c_double),
        ("order", C.c_int),
        ("CFL", C.c_double),
        ("ic", C.c_double * 4),
        ("localTimestep", C.c_int),
        ("multistageLimiting", C.c_int),
        ("cflAdjust", C.c_int),
        ("viscosity", C.c_int),
        ("Pr", C.c_double),
        ("R", C.c_double),
        ("mu", C.c_double),
        ("Re", C.c_double),
        ("L", C.c_double),
        ("mms", C.c_int),
        ("nbc", C.c_int),
        ("bcType", C.c_int * MAX_BC),
        ("bcNData", C.c_int * MAX_BC),
        ("bcData", (C.c_double * 4) * MAX_BC),
        ("nForceGroups", C.c_int),
        ("forceGroups", C.c_int * MAX_BC),
    ]


def build(force=False):
    """Compile oracle.c into oracle/_build/liboracle.so (strict IEEE: no FMA contraction)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-std=gnu11", "-fopenmp",
           "-o", tmp, SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.o_mesh_create.restype = C.c_void_p
        L.o_mesh_create.argtypes = [C.c_int, dp, C.c_int, ip, ip, C.c_int, ip, C.c_int, ip, ip]
        L.o_mesh_free.argtypes = [C.c_void_p]
        L.o_mesh_sizes.argtypes = [C.c_void_p, ip]
        L.o_mesh_geometry.argtypes = [C.c_void_p, dp, dp, ip, dp]
        L.o_setup.argtypes = [C.c_void_p, C.POINTER(OCfg)]
        L.o_get_state.argtypes = [C.c_void_p, dp]
        L.o_set_state.argtypes = [C.c_void_p, dp]
        L.o_get_cfg.argtypes = [C.c_void_p, C.POINTER(OCfg)]
        L.o_residual.argtypes = [C.c_void_p, dp, dp, dp, dp, C.c_int, C.c_int]
        L.o_residual.restype = C.c_int
        L.o_step.argtypes = [C.c_void_p, dp, dp]
        L.o_step.restype = C.c_int
        L.o_run.argtypes = [C.c_void_p, C.c_int, dp, ip]
        L.o_run.restype = C.c_int
        L.o_ms_converge.argtypes = [C.c_void_p, C.c_long, C.c_double, dp, dp]
        L.o_ms_converge.restype = C.c_long
        L.o_face_states.argtypes = [C.c_void_p, dp]
        L.o_grad_lim.argtypes = [C.c_void_p, dp, dp]
        L.o_edge_fluxes.argtypes = [C.c_void_p, dp]
        L.o_fallback_counts.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
        L.o_reconstruct.argtypes = [C.c_void_p, dp, ip]
        L.o_reconstruct.restype = C.c_int
        L.o_flux_batch.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, dp]
        L.o_diffusive_flux.argtypes = [C.c_double, C.c_double, dp, dp, dp, dp]
        L.o_mms_eval.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, C.POINTER(OCfg)]
        L.o_time.argtypes = [C.c_void_p]
        L.o_time.restype = C.c_double
        L.o_dt.argtypes = [C.c_void_p]
        L.o_dt.restype = C.c_double
        L.o_err_index.argtypes = [C.c_void_p]
        L.o_err_index.restype = C.c_long
        L.o_set_threads.argtypes = [C.c_int]
        L.o_max_threads.restype = C.c_int
        L.o_step.argtypes = [C.c_void_p, dp, dp]
        L.o_set_threads(1)
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def make_cfg(conf, mms=0, b_tags=None):
    """Fill an OCfg from a config dict produced by gmsh_ref.load_config."""
    c = OCfg()
    c.dt = conf["dt"]
    c.dynamicDt = int(conf["dynamicDt"])
    c.tEnd = conf["tEnd"]
    c.flux = gmsh_ref.FLUXES[conf["flux"]]
    c.integrator = gmsh_ref.INTEGRATORS[conf["integrator"]]
    c.limited = int(conf["limited"])
    c.lpThresh = conf["lpThresh"]
    c.order = conf["order"]
    c.CFL = conf["CFL"]
    for k in range(4):
        c.ic[k] = conf["ic"][k]
    c.localTimestep = int(conf["localTimestep"])
    c.multistageLimiting = int(conf["multistageLimiting"])
    c.cflAdjust = int(conf["cflAdjust"])
    c.viscosity = int(conf["viscosity"])
    pc = conf["physicalConfig"]
    c.Pr, c.R, c.Re, c.L = pc["Pr"], pc["R"], pc["Re"], pc["L"]
    c.mu = float("nan")
    c.mms = mms
    c.nbc = len(conf["boundaries"])
    for i, b in enumerate(conf["boundaries"]):
        c.bcType[i] = b["type"]
        c.bcNData[i] = len(b["q"])
        for k, v in enumerate(b["q"][:4]):
            c.bcData[i][k] = v
    fg = []
    if b_tags is not None:
        for t in conf["forceBoundary"]:
            if t in b_tags:
                fg.append(b_tags.index(t))
    c.nForceGroups = len(fg)
    for i, g in enumerate(fg):
        c.forceGroups[i] = g
    return c


class OracleMesh:
    """One mesh + config in the oracle (mirrors UMesh2 after buildMesh + ufvmSetup)."""

    def __init__(self, mesh, conf, mms=0):
        L = lib()
        self.mesh = mesh
        self.conf = conf
        nodes = np.ascontiguousarray(mesh["nodes"][:, :2], dtype=np.float64)
        els = mesh["elements"]
        off = np.zeros(len(els) + 1, dtype=np.int32)
        off[1:] = np.cumsum([len(e) for e in els])
        en = np.ascontiguousarray(np.concatenate([np.asarray(e, dtype=np.int32) for e in els]), dtype=np.int32)
        bn = np.ascontiguousarray(np.asarray(mesh["bNodes"], dtype=np.int32).reshape(-1, 2))
        bgs = np.asarray(mesh["bGroupStart"], dtype=np.int32)
        tags = [b["tag"] for b in conf["boundaries"]]
        gbc = []
        for t in mesh["bTags"]:
            if t not in tags:
                raise ValueError("Could not find matching boundary condition tag " + t)
            gbc.append(tags.index(t))
        gbc = np.asarray(gbc, dtype=np.int32)
        self._keep = (nodes, off, en, bn, bgs, gbc)
        self.h = L.o_mesh_create(len(nodes), _dp(nodes), len(els), _ip(off), _ip(en), len(bn), _ip(bn),
                                 len(bgs), _ip(bgs), _ip(gbc))
        sz = np.zeros(6, dtype=np.int32)
        L.o_mesh_sizes(self.h, _ip(sz))
        self.n_cells, self.n_ghost, self.n_edges, self.n_int, self.n_bnd, err = [int(x) for x in sz]
        if err != 0:
            raise ValueError("non-positive cell area")
        self.cfg = make_cfg(conf, mms, mesh["bTags"])
        L.o_setup(self.h, C.byref(self.cfg))

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().o_mesh_free(self.h)
                self.h = None
        except Exception:
            pass

    def geometry(self):
        L = lib()
        cg = np.zeros((self.n_cells, 18))
        eg = np.zeros((self.n_edges, 8))
        ct = np.zeros((self.n_cells, 18), dtype=np.int32)
        gc = np.zeros((self.n_ghost, 2))
        L.o_mesh_geometry(self.h, _dp(cg), _dp(eg), _ip(ct), _dp(gc))
        return {"cell": cg, "edge": eg, "topo": ct, "ghost_centroid": gc}

    def state(self):
        q = np.zeros((self.n_cells, 4))
        lib().o_get_state(self.h, _dp(q))
        return q

    def set_state(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        lib().o_set_state(self.h, _dp(q))

    def residual(self, q, limit=True, dt_update=True):
        """One ufvmSolver call (plus the MMS source when mms != 0) on q[n_cells,4]."""
        qq = np.zeros((self.n_cells + self.n_ghost, 4))
        qq[:self.n_cells] = q
        R = np.zeros_like(qq)
        nd = np.zeros(1)
        rm = np.zeros(1)
        st = lib().o_residual(self.h, _dp(qq), _dp(R), _dp(nd), _dp(rm), int(limit), int(dt_update))
        if st:
            raise RuntimeError("oracle residual failed with status %d at index %d" % (st, lib().o_err_index(self.h)))
        return R[:self.n_cells].copy(), float(nd[0]), float(rm[0])

    def run(self, nsteps):
        rec = np.zeros((nsteps, 9))
        done = C.c_int(0)
        st = lib().o_run(self.h, nsteps, _dp(rec), C.byref(done))
        if st:
            raise RuntimeError("oracle run failed with status %d at index %d" % (st, lib().o_err_index(self.h)))
        return rec[:done.value].copy()

    def face_states(self):
        n = sum(len(e) for e in self.mesh["elements"])
        out = np.zeros((n, 4))
        lib().o_face_states(self.h, _dp(out))
        return out

    def edge_fluxes(self):
        """len * flux of every edge (reference edge order) of the last residual evaluation."""
        out = np.zeros((self.n_edges, 4))
        lib().o_edge_fluxes(self.h, _dp(out))
        return out

    def fallback_counts(self):
        """(interior, boundary) faces whose reconstruction took the negative-pressure
        fallback in the last residual evaluation."""
        out = (C.c_long * 2)()
        lib().o_fallback_counts(self.h, out)
        return int(out[0]), int(out[1])

    def grad_lim(self):
        g = np.zeros((self.n_cells, 4, 2))
        l = np.zeros((self.n_cells, 4, 2))
        lib().o_grad_lim(self.h, _dp(g), _dp(l))
        return g, l

    def reconstruct(self):
        """ebb-reconstruct values (reconstruct.d:79-424): (node values, edge values, cell
        averages) as three (n, 4) arrays."""
        n_nodes = len(self.mesh["nodes"])
        out = np.zeros((n_nodes + self.n_edges + self.n_cells, 4))
        cnt = np.zeros(3, dtype=np.int32)
        st = lib().o_reconstruct(self.h, _dp(out), _ip(cnt))
        if st:
            raise RuntimeError("oracle reconstruct failed with status %d at index %d" % (st, lib().o_err_index(self.h)))
        a, b, c = (int(x) for x in cnt)
        return out[:a].copy(), out[a:a + b].copy(), out[a + b:a + b + c].copy()

    def ms_converge(self, max_iter, tol=1e-10):
        l2 = np.zeros(4)
        rm = np.zeros(1)
        it = lib().o_ms_converge(self.h, max_iter, tol, _dp(l2), _dp(rm))
        return int(it), l2, float(rm[0])

    @property
    def t(self):
        return lib().o_time(self.h)

    @property
    def dt(self):
        return lib().o_dt(self.h)


def set_threads(n):
    """Threads of the oracle's parallel loops (1 = the sequential reference order)."""
    lib().o_set_threads(int(n))


def max_threads():
    return lib().o_max_threads()


def flux_batch(kind, qL, qR, n):
    qL = np.ascontiguousarray(qL, dtype=np.float64).reshape(-1, 4)
    qR = np.ascontiguousarray(qR, dtype=np.float64).reshape(-1, 4)
    n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1, 2)
    F = np.zeros_like(qL)
    s = np.zeros(len(qL))
    lib().o_flux_batch(int(kind), len(qL), _dp(qL), _dp(qR), _dp(n), _dp(F), _dp(s))
    return F, s


def diffusive_flux(Pr, mu, q, dq, n):
    q = np.ascontiguousarray(q, dtype=np.float64)
    dq = np.ascontiguousarray(dq, dtype=np.float64).reshape(4, 2)
    n = np.ascontiguousarray(n, dtype=np.float64)
    out = np.zeros(4)
    lib().o_diffusive_flux(Pr, mu, _dp(q), _dp(dq), _dp(n), _dp(out))
    return out


def mms_eval(kind, xy, cfg=None):
    xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
    n = len(xy)
    q = np.zeros((n, 4))
    g = np.zeros((n, 4, 2))
    s = np.zeros((n, 4))
    if cfg is None:
        cfg = OCfg()
    lib().o_mms_eval(int(kind), n, _dp(xy), _dp(q), _dp(g), _dp(s), C.byref(cfg))
    return q, g, s
