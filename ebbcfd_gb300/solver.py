"""Python face of the GB300 solver, mirroring the reference's operator interface.

Names follow EbbCFD's D modules:
  load_config            source/config.d:112 loadConfig
  import_mesh            source/io.d:669 importMesh
  UfvmSolver.ufvm_solver source/solve.d:322 ufvmSolver!(F,4)(R, q, mesh, config, newDt, Rmax, limit, dtUpdate)
  UfvmSolver.step        source/integrators.d Euler/RK2/RK2_TVD/RK4 .step!solver
  UfvmSolver.run         app/solver.d:38 runIntegrator loop body
  roe_flux / rusanov_flux  source/flux.d:224 / :66
  save_solution / load_solution  source/io.d:68 / :218

Every call goes through the C ABI of include/ebb_gb300.h into the CUDA library; there
is no CPU path.  Failures raise EbbError (EdgeException / CellException for the NaN
checks the reference reports with those exception types).
"""
import ctypes as C

import numpy as np

from . import _lib

PRECISION = {"fp64": 0, "split": 1, "df": 2}
FLUX = {"rusanovFlux": 0, "roeFlux": 1}
INTEGRATOR = {"Euler": 0, "RK2": 1, "RK2_TVD": 2, "RK4": 3}
BC = {"fullState": 0, "constP": 1, "inviscidWall": 2, "viscidWall": 3, "symmetry": 4, "tpInflow": 5, "dirichlet": 6}


class EbbError(RuntimeError):
    def __init__(self, code, msg, index=-1):
        super().__init__("%s (%d): %s%s" % (_lib.STATUS.get(code, "?"), code, msg,
                                            "" if index < 0 else " [index %d]" % index))
        self.code = code
        self.index = index


class EdgeException(EbbError):
    """NaN face flux (solve.d:805-806 and siblings); index is the reference edge id."""


class CellException(EbbError):
    """NaN cell state after a step (app/solver.d:131-149); index is the reference cell id."""


def _check(code, msg="", index=-1):
    if code == 0:
        return
    if code == 8:
        raise EdgeException(code, msg or "Got NaN on edge", index)
    if code == 9:
        raise CellException(code, msg or "Got nan on cell average value", index)
    raise EbbError(code, msg, index)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def load_config(text):
    """Parse ebb-solve JSON (config.d semantics) into the C config struct."""
    L = _lib.load()
    cfg = _lib.Config()
    err = C.create_string_buffer(512)
    _check(L.ebb_config_parse(text.encode(), C.byref(cfg), err, 512), err.value.decode())
    return cfg


def default_config():
    cfg = _lib.Config()
    _lib.load().ebb_config_defaults(C.byref(cfg))
    return cfg


def set_boundaries(cfg, bcs):
    """bcs: list of (tag, type-name, [data...])."""
    cfg.n_boundaries = len(bcs)
    for i, (tag, typ, data) in enumerate(bcs):
        b = cfg.boundaries[i]
        b.tag = tag.encode()
        b.type = BC[typ] if isinstance(typ, str) else int(typ)
        b.n_data = len(data)
        for k, v in enumerate(data):
            b.data[k] = float(v)
    return cfg


def set_force_boundary(cfg, tags):
    cfg.n_force = len(tags)
    for i, t in enumerate(tags):
        cfg.force_boundary[i].value = t.encode()
    return cfg


class Mesh:
    """A gmsh mesh as the reference reads it (nodes, elements, boundary groups)."""

    def __init__(self, handle):
        self.h = handle
        self._info = None

    @classmethod
    def from_arrays(cls, nodes, elements, b_nodes, b_group_start, tags):
        """nodes (N,2); elements: list of 1-based node lists or (M,k) array; b_nodes (B,2) 0-based."""
        L = _lib.load()
        xy = np.ascontiguousarray(np.asarray(nodes, dtype=np.float64)[:, :2])
        if isinstance(elements, np.ndarray) and elements.ndim == 2:
            off = np.arange(0, elements.size + 1, elements.shape[1], dtype=np.int64)
            en = np.ascontiguousarray(elements.reshape(-1), dtype=np.int32)
        else:
            lens = [len(e) for e in elements]
            off = np.zeros(len(elements) + 1, dtype=np.int64)
            off[1:] = np.cumsum(lens)
            en = np.ascontiguousarray(np.concatenate([np.asarray(e, dtype=np.int32) for e in elements]))
        bn = np.ascontiguousarray(np.asarray(b_nodes, dtype=np.int32).reshape(-1, 2))
        bgs = np.ascontiguousarray(np.asarray(b_group_start, dtype=np.int64))
        tb = b"".join(t.encode().ljust(_lib.TAG_LEN, b"\0")[:_lib.TAG_LEN] for t in tags)
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        code = L.ebb_mesh_from_arrays(len(xy), _dp(xy), len(off) - 1, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                      en.ctypes.data_as(C.POINTER(C.c_int32)), len(bn),
                                      bn.ctypes.data_as(C.POINTER(C.c_int32)), len(tags),
                                      bgs.ctypes.data_as(C.POINTER(C.c_int64)), tb, C.byref(h), err, 512)
        _check(code, err.value.decode())
        return cls(h)

    @property
    def info(self):
        if self._info is None:
            inf = _lib.MeshInfo()
            _check(_lib.load().ebb_mesh_get_info(self.h, C.byref(inf)))
            self._info = inf
        return self._info

    @property
    def n_cells(self):
        return self.info.n_cells

    @property
    def tags(self):
        L = _lib.load()
        out = []
        for i in range(self.info.n_tags):
            b = C.create_string_buffer(_lib.TAG_LEN)
            L.ebb_mesh_get_tag(self.h, i, b, _lib.TAG_LEN)
            out.append(b.value.decode())
        return out

    def centroids(self):
        xy = np.zeros((self.n_cells, 2))
        _check(_lib.load().ebb_mesh_centroids(self.h, _dp(xy)))
        return xy

    def edges(self):
        """The reference's edges in creation order: dict of group (boundary tag index, -1
        interior), cells (n, 2), mid (n, 2), normal (n, 2), len (n,)."""
        n = self.info.n_edges
        g = np.zeros(n, dtype=np.int32)
        c = np.zeros((n, 2), dtype=np.int32)
        mid = np.zeros((n, 2))
        nrm = np.zeros((n, 2))
        ln = np.zeros(n)
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        _check(_lib.load().ebb_mesh_edges(self.h, ip(g), ip(c), _dp(mid), _dp(nrm), _dp(ln)))
        return {"group": g, "cells": c, "mid": mid, "normal": nrm, "len": ln}

    def __del__(self):
        try:
            if self.h:
                _lib.load().ebb_mesh_free(self.h)
                self.h = None
        except Exception:
            pass


def import_mesh(path):
    L = _lib.load()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    _check(L.ebb_mesh_import(str(path).encode(), C.byref(h), err, 512), err.value.decode())
    return Mesh(h)


class UfvmSolver:
    """Device-resident solver for one mesh + config (buildMesh + ufvmSetup)."""

    n = 1  # instances in the arena

    def __init__(self, mesh, cfg, precision="fp64"):
        L = _lib.load()
        self.mesh = mesh
        self.cfg = cfg
        self.n_cells = mesh.n_cells
        self.face_slots = mesh.info.face_slots
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        code = L.ebb_solver_create(mesh.h, C.byref(cfg), PRECISION[precision], C.byref(h), err, 512)
        _check(code, err.value.decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            _lib.load().ebb_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _raise(self, code):
        if code == 0:
            return
        L = _lib.load()
        kind = C.c_int32()
        idx = C.c_int64()
        msg = C.create_string_buffer(256)
        L.ebb_last_error(self.h, C.byref(kind), C.byref(idx), msg, 256)
        _check(code, msg.value.decode(), idx.value)

    @property
    def state(self):
        q = np.zeros((self.n_cells, 4))
        self._raise(_lib.load().ebb_get_state(self.h, _dp(q)))
        return q

    def set_state(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.n_cells, 4)
        self._raise(_lib.load().ebb_set_state(self.h, _dp(q)))

    def time(self):
        t = C.c_double()
        dt = C.c_double()
        it = C.c_int64()
        self._raise(_lib.load().ebb_get_time(self.h, C.byref(t), C.byref(dt), C.byref(it)))
        return t.value, dt.value, it.value

    def set_time(self, t, dt):
        self._raise(_lib.load().ebb_set_time(self.h, float(t), float(dt)))

    def ufvm_solver(self, q, limit=True, dt_update=True, rmax=0.0):
        """One residual evaluation; returns (R, newDt, Rmax)."""
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.n_cells, 4)
        R = np.zeros_like(q)
        nd = C.c_double()
        rm = C.c_double(rmax)
        self._raise(_lib.load().ebb_residual(self.h, _dp(q), _dp(R), C.byref(nd), C.byref(rm), int(limit),
                                             int(dt_update)))
        return R, nd.value, rm.value

    def step(self, dt, rmax=0.0):
        """One integrator step on the resident state; returns (next dt, Rmax)."""
        d = C.c_double(dt)
        rm = C.c_double(rmax)
        self._raise(_lib.load().ebb_step(self.h, C.byref(d), C.byref(rm)))
        return d.value, rm.value

    def run(self, nsteps, records=True):
        """Up to nsteps runIntegrator iterations; returns an (n, 11) array of
        (t, drag, lift, resid_rho, resid_u, resid_v, resid_E, Rmax, dt, cfl) rows + step count."""
        L = _lib.load()
        n = C.c_int64()
        if records:
            rec = (_lib.StepRecord * max(1, nsteps))()
            self._raise(L.ebb_run(self.h, int(nsteps), rec, C.byref(n)))
            arr = np.frombuffer(rec, dtype=np.float64).reshape(-1, 10)[:n.value].copy()
            return arr
        self._raise(L.ebb_run(self.h, int(nsteps), None, C.byref(n)))
        return n.value

    def face_states(self):
        out = np.zeros((self.face_slots, 4))
        self._raise(_lib.load().ebb_get_face_states(self.h, _dp(out)))
        return out

    def edge_fluxes(self):
        """len * flux of every edge (reference edge order) of the last residual evaluation."""
        out = np.zeros((self.mesh.info.n_edges, 4))
        self._raise(_lib.load().ebb_get_edge_fluxes(self.h, _dp(out)))
        return out

    def save_solution(self, path, t=None, dt=None):
        """io.d:68 saveSolution; t and dt default to the solver's current time and step."""
        if t is None or dt is None:
            t0, dt0, _ = self.time()
            t = t0 if t is None else t
            dt = dt0 if dt is None else dt
        self._raise(_lib.load().ebb_save_solution(self.h, str(path).encode(), float(t), float(dt)))

    def load_solution(self, path):
        self._raise(_lib.load().ebb_load_solution(self.h, str(path).encode()))

    def load_solution_parts(self, paths):
        """loadSolution of every rank's file of a partitioned run (cells by global id)."""
        arr = (C.c_char_p * len(paths))(*[str(p).encode() for p in paths])
        self._raise(_lib.load().ebb_load_solution_parts(self.h, len(paths), arr))

    def reconstruct(self, mmsh_path=None, esln_path=None, t=None, dt=None):
        """ebb-reconstruct (app/reconstruct.d:79-424) of the resident state: returns the
        (n, 4) values of the refined mesh (used nodes, edge midpoints, cells) and writes
        the .mmsh / .esln files when paths are given."""
        L = _lib.load()
        n = C.c_int64()
        self._raise(L.ebb_reconstruct(self.h, self.mesh.h, None, None, 0.0, 0.0, None, C.byref(n)))
        if t is None or dt is None:
            t0, dt0, _ = self.time()
            t = t0 if t is None else t
            dt = dt0 if dt is None else dt
        q = np.zeros((n.value, 4))
        self._raise(L.ebb_reconstruct(self.h, self.mesh.h, None if mmsh_path is None else str(mmsh_path).encode(),
                                      None if esln_path is None else str(esln_path).encode(), float(t), float(dt),
                                      _dp(q), C.byref(n)))
        return q

    def status(self, first=0, count=None):
        """list of dicts (cell_offset, n_cells, iterations, t, dt, cfl, done, status, err_index,
        drag, lift, resid, rmax, resid_first) for instances first..first+count-1"""
        count = self.n - first if count is None else count
        arr = (_lib.InstanceStatus * max(1, count))()
        self._raise(_lib.load().ebb_batch_status(self.h, first, count, arr))
        out = []
        for k in range(count):
            d = {f: getattr(arr[k], f) for f in STATUS_FIELDS}
            d["resid"] = list(d["resid"])
            out.append(d)
        return out

    def set_stop(self, k=-1, t_end=1e300, max_steps=0, resid_drop=0.0):
        self._raise(_lib.load().ebb_batch_set_stop(self.h, int(k), float(t_end), int(max_steps), float(resid_drop)))


def _flux(kind, qL, qR, n):
    L = _lib.load()
    qL = np.ascontiguousarray(qL, dtype=np.float64).reshape(-1, 4)
    qR = np.ascontiguousarray(qR, dtype=np.float64).reshape(-1, 4)
    n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1, 2)
    F = np.zeros_like(qL)
    s = np.zeros(len(qL))
    _check(L.ebb_flux(kind, len(qL), _dp(qL), _dp(qR), _dp(n), _dp(F), _dp(s)))
    return F, s


def roe_flux(qL, qR, n):
    return _flux(1, qL, qR, n)


def rusanov_flux(qL, qR, n):
    return _flux(0, qL, qR, n)


def _mesh_cfg_arrays(meshes, cfgs):
    if isinstance(cfgs, _lib.Config):
        cfgs = [cfgs] * len(meshes)
    if len(cfgs) != len(meshes) or not meshes:
        raise ValueError("one config per mesh is needed")
    mh = (C.c_void_p * len(meshes))(*[m.h.value if isinstance(m.h, C.c_void_p) else m.h for m in meshes])
    ca = (_lib.Config * len(cfgs))(*cfgs)
    return mh, ca


def batch_footprint(meshes, cfgs, precision="fp64"):
    """Device bytes an arena of these solves takes (host-side layout only, no GPU)."""
    mh, ca = _mesh_cfg_arrays(meshes, cfgs)
    out = C.c_size_t()
    err = C.create_string_buffer(512)
    _check(_lib.load().ebb_batch_footprint(len(meshes), mh, ca, PRECISION[precision], C.byref(out), err, 512),
           err.value.decode())
    return out.value


STATUS_FIELDS = [f[0] for f in _lib.InstanceStatus._fields_]


class UfvmBatch(UfvmSolver):
    """Many independent solves (mesh + config each) in one device arena, advanced
    together by the same kernel launches; every instance stops at its own tEnd, step
    limit or residual drop, and a NaN halts only its own instance."""

    def __init__(self, meshes, cfgs, precision="fp64"):
        L = _lib.load()
        mh, ca = _mesh_cfg_arrays(meshes, cfgs)
        self.meshes = list(meshes)
        self.cfg = ca[0]
        self.n = len(meshes)
        self.n_cells = sum(m.n_cells for m in meshes)
        self.face_slots = sum(m.info.face_slots for m in meshes)
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        _check(L.ebb_batch_create(self.n, mh, ca, PRECISION[precision], C.byref(h), err, 512), err.value.decode())
        self.h = h

    def instance_state(self, k):
        q = np.zeros((self.meshes[k].n_cells, 4))
        self._raise(_lib.load().ebb_batch_get_state(self.h, int(k), _dp(q)))
        return q

    def set_instance_state(self, k, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.meshes[k].n_cells, 4)
        self._raise(_lib.load().ebb_batch_set_state(self.h, int(k), _dp(q)))

    def launch(self, nsteps):
        """enqueue nsteps iterations on the arena's stream without waiting"""
        self._raise(_lib.load().ebb_launch_steps(self.h, int(nsteps)))

    def sync(self):
        self._raise(_lib.load().ebb_sync(self.h))


RESULT_FIELDS = [f[0] for f in _lib.RequestResult._fields_]


class EbbServer:
    """Continuous-batching request loop (include/ebb_gb300.h ebb_server_*): submit solves
    at any time, call tick() to run scheduling rounds, collect finished results."""

    def __init__(self, precision="split", **options):
        L = _lib.load()
        o = _lib.ServerOptions()
        L.ebb_server_options_defaults(C.byref(o))
        o.precision = PRECISION[precision]
        for k, v in options.items():
            setattr(o, k, PRECISION[v] if k == "finish_precision" and isinstance(v, str) else v)
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        _check(L.ebb_server_create(C.byref(o), C.byref(h), err, 512), err.value.decode())
        self.h = h
        self.options = o
        self.n_cells = {}

    def submit(self, mesh, cfg, max_steps=0, resid_drop=0.0):
        i = C.c_int64()
        _check(_lib.load().ebb_server_submit(self.h, mesh.h, C.byref(cfg), int(max_steps), float(resid_drop),
                                             C.byref(i)))
        self.n_cells[i.value] = mesh.n_cells
        return i.value

    def tick(self):
        a = C.c_int32()
        w = C.c_int32()
        _check(_lib.load().ebb_server_tick(self.h, C.byref(a), C.byref(w)))
        return a.value, w.value

    def results(self):
        out = []
        buf = (_lib.RequestResult * 256)()
        n = C.c_int32()
        while True:
            _check(_lib.load().ebb_server_results(self.h, buf, 256, C.byref(n)))
            for k in range(n.value):
                d = {f: getattr(buf[k], f) for f in RESULT_FIELDS}
                d["resid"] = list(d["resid"])
                d["msg"] = d["msg"].decode(errors="replace")
                out.append(d)
            if n.value < 256:
                return out

    def take_state(self, rid):
        q = np.zeros((self.n_cells[rid], 4))
        _check(_lib.load().ebb_server_take_state(self.h, int(rid), _dp(q)))
        return q

    def stats(self):
        s = _lib.ServerStats()
        _check(_lib.load().ebb_server_stats_get(self.h, C.byref(s)))
        return {f[0]: getattr(s, f[0]) for f in _lib.ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            _lib.load().ebb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
