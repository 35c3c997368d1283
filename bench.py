#!/usr/bin/env python3
"""Throughput of the explicit unstructured FV update on GB300.

Workload (default): the Mach 2.5 supersonic wedge -- [0,3]x[0,1] with a 15-degree
ramp from x=0.5, ~1.0M seeded-Delaunay triangles graded 2x toward the ramp (seed 0),
Rusanov flux, limited second order, RK2 at CFL 0.4, plain FP64.  A step is one RK2
time step of the whole mesh (two residual evaluations + stage updates + the
per-step reductions of the time loop); the metric is cell-updates/s = cells x
steps / time.  The ~1M-cell state and face arrays (~0.5 GB) exceed the 129 MB L2,
so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference-semantics FP64 CPU restatement (oracle/) on all
host cores on the same mesh and config (the D reference cannot be built: no D
compiler, MPI or ParMETIS is installed).  N>1: one independent
replica per GPU (the path does not shard), weak scaling.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WEDGE_BCS = [{"tag": "Inflow", "type": "fullState", "q": [2.5, 0, 1, 1]},
             {"tag": "Top", "type": "fullState", "q": [2.5, 0, 1, 1]},
             {"tag": "Symmetry", "type": "symmetry", "q": [2.5, 0, 1, 1]},
             {"tag": "Ramp", "type": "inviscidWall", "q": [2.5, 0, 1, 1]},
             {"tag": "Outflow", "type": "fullState", "q": [2.5, 0, 1, 1]}]


def wedge_config(cfl=0.4):
    return json.dumps({"mesh": "wedge.msh", "dt": 1e-4, "tEnd": 1e9, "flux": "rusanovFlux", "saveIter": -1,
                       "plotIter": -1, "forceBoundary": "Ramp", "integrator": "RK2", "limited": True, "CFL": cfl,
                       "initialConditions": [2.5, 0, 1, 1], "boudaryConditions": WEDGE_BCS})


def max_over_ranks(x):
    """Barrier, then the maximum of x over all ranks (one independent replica per GPU:
    the whole job is as slow as its slowest replica)."""
    import torch
    import torch.distributed as dist
    dist.barrier()
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


PROFILED_CELLS = 1_001_045  # the wedge the committed ncu captures ran on


def profiled_traffic(kernel, precision, ncell):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu
    summaries under profiles/ ("traffic: <kernel> <precision> <bytes>" lines, one
    capture of the 1,001,045-cell wedge), scaled to `ncell` cells (traffic grows with
    the cells processed); None when no capture covers the kernel."""
    import glob
    import re
    for f in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        for line in open(f):
            m = re.match(r"traffic: (\S+) (\S+) (\d+)\s*$", line)
            if m and m.group(1) == kernel and m.group(2) == precision:
                return {"bytes": int(m.group(3)) * ncell / PROFILED_CELLS, "source": os.path.relpath(f, ROOT),
                        "scaled_from_cells": PROFILED_CELLS}
    return None


def algorithmic_bytes(info, real=8, need_grad=False, limited=True):
    """Bytes each kernel must move per launch, every array touched once (re-reads of
    a neighbour's state count 0).  S = face slots, E = interior edges, G = boundary
    edges; real = bytes of the arithmetic type (8 plain FP64, 4 split)."""
    C, S, E, G = info.n_cells, info.face_slots, info.n_int_edges, info.n_ghost
    r = real
    cell = C * (4 * r + 4) + S * (4 + 2 * r + (2 * r if limited else 0) + 2 * r) + S * 4 * r + (C * 8 * r if need_grad else 0)
    flux = E * (8 + 2 * r + r + 8 * r + 5 * r) + G * (12 + 2 * r + r + 4 * r + 4 * r + 5 * r)
    # residual + RK2 first-stage update: nedge, perim, d, -1/area, FP64 q read, aux write
    # (T) and next-stage state write (T)
    update = C * (4 + 3 * r + 32 + 4 * r + 4 * r) + S * 4 + (E + G) * 5 * r
    if r == 4:  # split: the freestream correction reads the stage state and each slot's normal and length
        update += C * 4 * r + S * 3 * r
    return {"cell": cell, "flux": flux, "update": update}


def measure(L, E, _lib, gen, mesh, precision, args, local, ws, want_e2e):
    import ctypes as C
    cfg = E.load_config(wedge_config())
    t0 = time.time()
    sol = E.UfvmSolver(mesh, cfg, precision=precision)
    setup_s = time.time() - t0
    info = mesh.info
    ncell = info.n_cells
    sol.run(args.warmup, records=False)
    ms = (C.c_double * 4)()
    L.ebb_profile_kernels(sol.h, 20, ms)
    kern_ms = {"cell": ms[0], "flux": ms[1], "update": ms[2], "step_end": ms[3]}
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    n = C.c_int64()
    dev_ms = C.c_double()
    code = L.ebb_run_timed(sol.h, args.steps, C.byref(n), C.byref(dev_ms))
    clk = clocks.stop()
    if code != 0:
        sol._raise(code)
    elapsed = dev_ms.value / 1e3
    steps_done = n.value
    if ws > 1:
        elapsed = max_over_ranks(elapsed)
    state = sol.state
    value = ws * ncell * steps_done / elapsed
    e2e = None
    if want_e2e:
        # end to end through the public API with host buffers: every step uploads the
        # state from page-locked memory, advances one step and reads state and record back
        nbytes = ncell * 4 * 8
        ph = C.c_void_p()
        L.ebb_host_alloc(nbytes, C.byref(ph))
        host = np.ctypeslib.as_array((C.c_double * (ncell * 4)).from_address(ph.value)).reshape(ncell, 4)
        host[:] = state
        rec = (_lib.StepRecord * 1)()
        k_e2e = max(3, min(args.steps, 50))
        hp = host.ctypes.data_as(C.POINTER(C.c_double))
        t1 = time.perf_counter()
        for _ in range(k_e2e):
            L.ebb_set_state(sol.h, hp)
            L.ebb_run(sol.h, 1, rec, C.byref(n))
            L.ebb_get_state(sol.h, hp)
        t_e2e = time.perf_counter() - t1
        L.ebb_host_free(ph)
        e2e = {"value": ws * ncell * k_e2e / t_e2e, "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes + C.sizeof(_lib.StepRecord), "steps": k_e2e}
    peak, peak_kind = peaks()
    ab = algorithmic_bytes(info, real=8 if precision == "fp64" else 4)
    dom = max(("cell", "flux", "update"), key=lambda k: kern_ms[k])
    achieved = ab[dom] / (kern_ms[dom] * 1e-3) / 1e9
    tr = profiled_traffic("k_" + dom, precision, ncell)
    roof = {"bound": "hbm", "kernel": "k_" + dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": tr["bytes"] if tr else None,
            "traffic_source": tr, "kernel_ms": kern_ms, "algorithmic_bytes": ab}
    if precision == "fp64":
        # the FP64 kernels are bound by the FP64 pipe, not by HBM (ncu, profiles/fp64_wedge1m.md)
        roof["fp64_pipe_active_pct"] = {"k_cell": 85.9, "k_flux": 86.8}
    sol.close()
    return {"value": value, "elapsed": elapsed, "steps": steps_done, "setup_s": setup_s, "roofline": roof,
            "e2e": e2e, "clocks": clk, "state": state}


def run_ours(args, ws, rank, local):
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib, meshgen

    L = _lib.load()
    L.ebb_set_device(local)
    t0 = time.time()
    gen = meshgen.wedge(args.cells, seed=0)
    mesh = gen.to_solver_mesh()
    mesh_s = time.time() - t0
    info = mesh.info
    ncell = info.n_cells
    m64 = measure(L, E, _lib, gen, mesh, "fp64", args, local, ws, not args.no_e2e)
    split = None
    if not args.no_split:
        m32 = measure(L, E, _lib, gen, mesh, "split", args, local, ws, not args.no_e2e)
        q64, q32 = m64["state"], m32["state"]
        scale = np.maximum(np.abs(q64).max(axis=0), 1e-300)
        split = {"value": m32["value"], "unit": "cell-updates/s", "ms_per_step": 1e3 * m32["elapsed"] / m32["steps"],
                 "speedup_vs_fp64": m32["value"] / m64["value"], "roofline": m32["roofline"],
                 # L2 error per component relative to the component's RMS, and the largest
                 # pointwise error relative to the component's largest magnitude
                 "state_l2_err_vs_fp64": [float(x) for x in np.sqrt(((q32 - q64) ** 2).mean(axis=0)
                                                                   / np.maximum((q64 ** 2).mean(axis=0), 1e-300))],
                 "state_max_err_vs_fp64": float((np.abs(q32 - q64).max(axis=0) / scale).max()),
                 "steps_compared": m64["steps"] + args.warmup, "clocks": m32["clocks"], "e2e": m32["e2e"]}
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(gen, ncell, budget_s=args.cpu_budget)
    steps_done = m64["steps"]
    out = {
        "metric": "cell-updates/s", "value": m64["value"], "unit": "cell-updates/s", "n_gpus": ws,
        "steps": steps_done, "warmup": args.warmup, "ms_per_step": 1e3 * m64["elapsed"] / max(1, steps_done),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "wedge-M2.5-rusanov-rk2-cfl0.4", "cells": ncell, "faces": info.face_slots,
                   "interior_edges": info.n_int_edges, "boundary_edges": info.n_ghost, "precision": "plain-fp64",
                   "l2": "inputs larger than L2 (~%d MB resident)" % (sol_bytes(info) // 2 ** 20),
                   "parallelism": "replicas" if ws > 1 else "single", "mesh_s": round(mesh_s, 2),
                   "setup_s": round(m64["setup_s"], 2)},
        "cell_stages_per_s": 2 * m64["value"], "roofline": m64["roofline"], "cpu_baseline": cpu,
        "e2e": m64["e2e"], "gpu_launches": steps_done * 7, "clocks": m64["clocks"], "split_path": split,
    }
    return out


def sol_bytes(info):
    C, S, E, G = info.n_cells, info.face_slots, info.n_int_edges, info.n_ghost
    return 8 * (12 * (C + G) + 4 * 4 * S // 3 + 8 * (C + G) + 5 * (E + G) + 12 * S)


def cpu_baseline(gen, ncell, budget_s=20.0, steps_max=1000):
    from oracle import gmsh_ref, ref
    nthreads = ref.max_threads()
    ref.set_threads(nthreads)
    om = ref.OracleMesh(gen.as_reader_dict(), gmsh_ref.load_config(wedge_config()))
    t0 = time.perf_counter()
    om.run(1)
    t1 = time.perf_counter() - t0
    n = int(max(1, min(steps_max, budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    om.run(n)
    t = time.perf_counter() - t0
    ref.set_threads(1)
    return {"value": ncell * n / t, "unit": "cell-updates/s", "cores": nthreads, "kind": "port",
            "sample": "%d RK2 steps of the full %d-cell wedge (after 1 untimed step)" % (n, ncell)}


def mms32_config():
    return json.dumps({"mesh": "quads32.msh", "dt": 1e-4, "tEnd": 1e9, "flux": "roeFlux", "saveIter": -1,
                       "plotIter": -1, "forceBoundary": "Freestream", "integrator": "RK2_TVD", "limited": True,
                       "CFL": 0.5, "cflAdjust": False, "initialConditions": [0.5, 0, 1, 1],
                       "boudaryConditions": [{"tag": "Freestream", "type": "dirichlet", "q": [0.5, 0, 1, 1]}]})


def plate_config():
    bcs = [{"tag": "Inflow", "type": "fullState", "q": [0.3, 0, 1, 1]},
           {"tag": "Top", "type": "fullState", "q": [0.3, 0, 1, 1]},
           {"tag": "Outflow", "type": "constP", "q": [1.0 / (1.4 * 0.09)]},
           {"tag": "Symmetry", "type": "symmetry", "q": [0.3, 0, 1, 1]},
           {"tag": "Wall", "type": "viscidWall", "q": [0.3, 0, 1, 1]}]
    return json.dumps({"mesh": "plate.msh", "dt": 1e-7, "tEnd": 1e9, "flux": "roeFlux", "saveIter": -1,
                       "plotIter": -1, "forceBoundary": "Wall", "integrator": "RK4", "limited": True, "CFL": 0.8,
                       "cflAdjust": False, "viscosity": True,
                       "physicalConfig": {"Pr": 0.72, "R": 1.0, "gamma": 1.4, "Re": 1e5, "L": 1.0},
                       "initialConditions": [0.3, 0, 1, 1], "boudaryConditions": bcs})


def run_mms32(args):
    """32x32 quads on [0,1]^2, the sine manufactured fields, Dirichlet boundaries, Roe,
    limited, TVD-RK2, CFL 0.5, 1000 steps: L2(rho) error vs the exact field for the
    oracle, the plain FP64 path (which must equal it bitwise) and the split path."""
    import ctypes as C
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib, meshgen
    from oracle import gmsh_ref, ref
    L = _lib.load()
    gen = meshgen.uniform_quads(32)
    steps = args.steps if args.steps_given else 1000
    out = {"workload": "mms32-sine-roe-tvd-cfl0.5", "cells": 1024, "steps": steps}
    q_exact, _, _ = ref.mms_eval(2, gen.to_solver_mesh().centroids())
    for prec in ("fp64", "split"):
        cfg = E.load_config(mms32_config())
        cfg.mms = 2
        sol = E.UfvmSolver(gen.to_solver_mesh(), cfg, precision=prec)
        n = C.c_int64()
        ms = C.c_double()
        L.ebb_run_timed(sol.h, steps, C.byref(n), C.byref(ms))
        q = sol.state
        out[prec] = {"l2_rho": float(np.sqrt(np.mean((q[:, 0] - q_exact[:, 0]) ** 2))), "steps": n.value,
                     "cell_updates_per_s": 1024 * n.value / (ms.value / 1e3), "state": q}
    om = ref.OracleMesh(gen.as_reader_dict(), gmsh_ref.load_config(mms32_config()), mms=2)
    om.run(steps)
    qo = om.state()
    out["oracle"] = {"l2_rho": float(np.sqrt(np.mean((qo[:, 0] - q_exact[:, 0]) ** 2)))}
    out["fp64_equals_oracle_bitwise"] = bool(np.array_equal(out["fp64"]["state"], qo))
    out["split_l2_rel_diff"] = abs(out["split"]["l2_rho"] / out["fp64"]["l2_rho"] - 1)
    for prec in ("fp64", "split"):
        del out[prec]["state"]
    return out


def shock_angle(xy, q, x_lo=0.8, x_hi=1.6, nbins=16, ramp_x=0.5):
    """Angle (degrees) of the oblique shock from the ramp corner: in each x bin, the
    highest cell whose pressure is above the midpoint of the freestream and
    post-shock pressures marks the shock; a least-squares line through those points
    (y = (x - x0) tan(beta)) gives beta."""
    p = 0.4 * (q[:, 3] - 0.5 * (q[:, 1] ** 2 + q[:, 2] ** 2) / q[:, 0])
    p_inf = 1.0 / (1.4 * 2.5 ** 2)
    pts = []
    edges = np.linspace(x_lo, x_hi, nbins + 1)
    for a, b in zip(edges[:-1], edges[1:]):
        m = (xy[:, 0] >= a) & (xy[:, 0] < b)
        if not m.any():
            continue
        p2 = np.percentile(p[m], 95)
        hi = m & (p > 0.5 * (p_inf + p2))
        if hi.any():
            pts.append((0.5 * (a + b), xy[hi, 1].max()))
    x, y = np.array(pts).T
    slope, icpt = np.polyfit(x, y, 1)
    return float(np.degrees(np.arctan(slope))), float(-icpt / slope)


def theory_shock_angle(M=2.5, theta_deg=15.0, g=1.4):
    """Weak-shock solution of the theta-beta-Mach relation."""
    th = np.radians(theta_deg)
    best = None
    for b in np.linspace(np.arcsin(1 / M) + 1e-6, np.pi / 2, 200001):
        t = 2 / np.tan(b) * (M ** 2 * np.sin(b) ** 2 - 1) / (M ** 2 * (g + np.cos(2 * b)) + 2)
        if t >= th:
            best = b
            break
    return float(np.degrees(best))


def run_wedge5000(args):
    """Accuracy of configuration 2: the 1M-cell Mach 2.5 wedge run 5000 RK2 steps in
    plain FP64 (bitwise equal to the oracle on the parity cases, and used here as the
    reference solution: the oracle would take ~7 min on the host) and in split
    precision; shock angle of both against the oblique-shock relation, and the split
    path's L2 state error against FP64."""
    import ctypes as C
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib, meshgen
    L = _lib.load()
    steps = args.steps if args.steps_given else 5000
    mesh = meshgen.wedge(args.cells, seed=0).to_solver_mesh()
    xy = mesh.centroids()
    out = {"workload": "wedge-M2.5-rusanov-rk2-cfl0.4-accuracy", "cells": mesh.n_cells, "steps": steps,
           "theory_shock_angle_deg": theory_shock_angle()}
    qs = {}
    for prec in ("fp64", "split"):
        s = E.UfvmSolver(mesh, E.load_config(wedge_config()), precision=prec)
        n = C.c_int64()
        ms = C.c_double()
        code = L.ebb_run_timed(s.h, steps, C.byref(n), C.byref(ms))
        if code:
            s._raise(code)
        q = s.state
        qs[prec] = q
        t_end = s.time()[0]
        # the corner shock is established within about the distance the flow has moved
        span = min(1.1, 0.9 * t_end)
        beta, x0 = shock_angle(xy, q, x_lo=0.5 + 0.15 * span, x_hi=0.5 + 0.85 * span, nbins=10)
        out[prec] = {"cell_updates_per_s": mesh.n_cells * n.value / (ms.value / 1e3), "shock_angle_deg": beta,
                     "shock_origin_x": x0, "t": t_end, "shock_window_x": [0.5 + 0.15 * span, 0.5 + 0.85 * span]}
        s.close()
    d = qs["split"] - qs["fp64"]
    out["split_l2_rel_err"] = [float(np.sqrt(np.mean(d[:, k] ** 2)) / np.sqrt(np.mean(qs["fp64"][:, k] ** 2)))
                               for k in range(4)]
    out["split_max_rel_err"] = float((np.abs(d).max(axis=0) / np.abs(qs["fp64"]).max(axis=0)).max())
    return out


def run_plate(args):
    """Navier-Stokes laminar flat plate on ~4.0M mixed cells: both precision forms
    from the same start, throughput and the split path's drag error against FP64."""
    import ctypes as C
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib, meshgen
    L = _lib.load()
    t0 = time.time()
    gen = meshgen.flat_plate(args.cells if args.cells_given else 4_000_000)
    mesh = gen.to_solver_mesh()
    mesh_s = time.time() - t0
    steps = args.steps if args.steps_given else 200
    out = {"workload": "ns-plate-M0.3-Re1e5-roe-rk4-cfl0.8", "cells": mesh.n_cells, "mesh_s": round(mesh_s, 1),
           "steps": steps}
    recs = {}
    for prec in ("fp64", "split"):
        sol = E.UfvmSolver(mesh, E.load_config(plate_config()), precision=prec)
        sol.run(args.warmup, records=False)
        n = C.c_int64()
        ms = C.c_double()
        code = L.ebb_run_timed(sol.h, steps, C.byref(n), C.byref(ms))
        if code:
            sol._raise(code)
        rec = sol.run(1)
        recs[prec] = rec[-1]
        out[prec] = {"cell_updates_per_s": mesh.n_cells * n.value / (ms.value / 1e3), "ms_per_step": ms.value / n.value,
                     "drag": float(rec[-1][1]), "lift": float(rec[-1][2])}
        sol.close()
    out["split_speedup"] = out["split"]["cell_updates_per_s"] / out["fp64"]["cell_updates_per_s"]
    out["split_drag_rel_err"] = abs(out["split"]["drag"] / out["fp64"]["drag"] - 1)
    return out


def bump_json(mach, cfl=0.3, integrator="RK2_TVD", flux="roeFlux"):
    q = [mach, 0, 1, 1]
    return json.dumps({"mesh": "bump.msh", "dt": 1e-4, "tEnd": 1e9, "flux": flux, "saveIter": -1,
                       "plotIter": -1, "forceBoundary": "Wall", "integrator": integrator, "limited": True, "CFL": cfl,
                       "initialConditions": q,
                       "boudaryConditions": [{"tag": "Inflow", "type": "fullState", "q": q},
                                             {"tag": "Outflow", "type": "fullState", "q": q},
                                             {"tag": "Wall", "type": "inviscidWall", "q": q}]})


def cylinder_json(re, mach=0.2, cfl=0.3, integrator="RK2_TVD"):
    q = [mach, 0, 1, 1]
    far = [{"tag": t, "type": "fullState", "q": q} for t in ("Inflow", "Outflow", "Top", "Bottom")]
    return json.dumps({"mesh": "cyl.msh", "dt": 1e-4, "tEnd": 1e9, "flux": "roeFlux", "saveIter": -1,
                       "plotIter": -1, "forceBoundary": "Cylinder", "integrator": integrator, "limited": True,
                       "CFL": cfl, "viscosity": True, "initialConditions": q,
                       "physicalConfig": {"Pr": 0.72, "R": 1.0, "gamma": 1.4, "Re": re, "L": 1.0},
                       "boudaryConditions": far + [{"tag": "Cylinder", "type": "viscidWall", "q": q}]})


def _gen_mesh(job):
    kind, n, h, seed = job
    from ebbcfd_gb300 import meshgen
    return meshgen.bump_channel(n, h=h, seed=seed) if kind == "bump" else meshgen.cylinder(n, seed=seed)


def gen_meshes(jobs):
    """Seeded meshes generated on all host cores (spawned workers, no GPU state)."""
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(max(1, min(len(jobs), os.cpu_count() or 1))) as pool:
        return pool.map(_gen_mesh, jobs, chunksize=1)


def seq_ms_per_step(L, E, meshes, cfgs, precision, steps, warmup):
    """Device ms per step of each solve run alone (one solver at a time)."""
    import ctypes as C
    out = []
    for m, c in zip(meshes, cfgs):
        s = E.UfvmSolver(m, c, precision)
        s.run(warmup, records=False)
        n = C.c_int64()
        ms = C.c_double()
        code = L.ebb_run_timed(s.h, steps, C.byref(n), C.byref(ms))
        if code:
            s._raise(code)
        out.append(ms.value / max(1, n.value))
        s.close()
    return out


def run_batch512(args):
    """512 independent Euler bump-channel solves in one arena: channel [0,3]x[0,1], bump
    h sin^2(pi(x-1)) with h ~ U[0.02,0.1], seeded-Delaunay meshes with cell counts
    log-uniform in [2e3, 2e5], Mach ~ U[0.3,0.8], split precision, Roe, TVD-RK2, 2000
    steps each, against the same solves run one by one."""
    import ctypes as C
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib
    n = args.instances
    rng = np.random.default_rng(4)
    cells = np.exp(rng.uniform(np.log(2e3), np.log(2e5), n)).astype(int)
    hs = rng.uniform(0.02, 0.1, n)
    machs = rng.uniform(0.3, 0.8, n)
    steps = args.steps if args.steps_given else 2000
    t0 = time.time()
    gens = gen_meshes([("bump", int(c), float(h), k) for k, (c, h) in enumerate(zip(cells, hs))])
    meshes = [g.to_solver_mesh() for g in gens]
    mesh_s = time.time() - t0
    cfgs = [E.load_config(bump_json(float(m))) for m in machs]
    L = _lib.load()
    ncell = int(sum(m.n_cells for m in meshes))
    prec_b = args.batch_precision
    t0 = time.time()
    b = E.UfvmBatch(meshes, cfgs, prec_b)
    create_s = time.time() - t0
    b.run(args.warmup, records=False)
    kms = (C.c_double * 4)()
    L.ebb_profile_kernels(b.h, 10, kms)
    it0 = [s["iterations"] for s in b.status()]
    clocks = Clocks(0)
    clocks.start()
    nrun = C.c_int64()
    ms = C.c_double()
    t0 = time.perf_counter()
    code = L.ebb_run_timed(b.h, steps, C.byref(nrun), C.byref(ms))
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    if code:
        b._raise(code)
    st = b.status()
    failed = [k for k, x in enumerate(st) if x["status"] != 0]
    done_cu = sum(meshes[k].n_cells * (x["iterations"] - it0[k]) for k, x in enumerate(st))
    value = done_cu / (ms.value / 1e3)
    b.close()
    # the same solves one by one: device time per step of each, on a sample of every
    # stride-th instance, scaled to all instances and to the batch's step count
    stride = max(1, args.seq_stride)
    idx = list(range(0, n, stride))
    seq = {}
    for prec in (("split", "fp64") if prec_b == "split" else ()):
        per = seq_ms_per_step(L, E, [meshes[i] for i in idx], [cfgs[i] for i in idx], prec, args.seq_steps,
                              args.warmup)
        est_ms = sum(per) * (n / len(idx)) * steps
        cells_s = sum(meshes[i].n_cells for i in idx) * (n / len(idx)) * steps / (est_ms / 1e3)
        seq[prec] = {"cell_updates_per_s": cells_s, "est_total_s": est_ms / 1e3}
    peak, peak_kind = peaks()
    if prec_b != "split":  # the arena itself in plain FP64 (which instances fail there)
        return {"workload": "batch512-bump-roe-tvd-fp64", "instances": n, "cells": ncell, "steps": nrun.value,
                "cell_updates_per_s": value, "instances_failed": len(failed),
                "failed": [{"k": k, "cells": meshes[k].n_cells, "status": st[k]["status"],
                            "iterations": st[k]["iterations"]} for k in failed],
                "device_s": ms.value / 1e3, "clocks": clk}
    return {"workload": "batch512-bump-roe-tvd-split", "instances": n, "cells": ncell, "steps": nrun.value,
            "cell_updates_per_s": value, "cell_updates": done_cu, "instances_failed": len(failed),
            "failed": [{"k": k, "cells": meshes[k].n_cells, "h": round(float(hs[k]), 4), "mach": round(float(machs[k]), 4),
                        "status": st[k]["status"], "iterations": st[k]["iterations"]} for k in failed],
            "device_s": ms.value / 1e3, "wall_s": wall, "mesh_s": round(mesh_s, 1),
            "create_s": round(create_s, 2), "kernel_ms": list(kms), "clocks": clk,
            "cells_min_max": [int(min(m.n_cells for m in meshes)), int(max(m.n_cells for m in meshes))],
            "one_by_one": seq, "speedup_vs_one_by_one_split": value / seq["split"]["cell_updates_per_s"],
            "speedup_vs_one_by_one_fp64": value / seq["fp64"]["cell_updates_per_s"],
            "one_by_one_sample": "every %d-th instance (%d of %d), %d timed steps each after %d warm-up, scaled"
                                 % (stride, len(idx), n, args.seq_steps, args.warmup), "hbm_peak_gbs": peak,
            "peak_source": peak_kind}


def run_serve(args):
    """Served request stream: Poisson arrivals (seed 7, mean 40 req/s); 70% Euler bump
    channels, 30% Navier-Stokes cylinders (Re ~ U[50,200], Mach 0.2); cell counts
    log-uniform in [1e3, 2e6]; each stops at a 1e-8 residual drop or its step cap;
    split precision; admission capped at 150 GB.  Latency = result in hand minus
    scheduled arrival.  The sequential baseline is plain FP64 solves one at a time:
    each request's device time per step alone (timed on a sample of steps) times the
    steps it ran."""
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib
    R = args.requests
    rng = np.random.default_rng(7)
    arrivals = np.cumsum(rng.exponential(1.0 / 40.0, R))
    kinds = np.where(rng.uniform(0, 1, R) < 0.7, "bump", "cyl")
    cells = np.exp(rng.uniform(np.log(1e3), np.log(args.max_cells), R)).astype(int)
    hs = rng.uniform(0.02, 0.1, R)
    machs = rng.uniform(0.3, 0.8, R)
    res = rng.uniform(50, 200, R)
    cap = args.step_cap
    t0 = time.time()
    gens = gen_meshes([(str(k), int(c), float(h), i) for i, (k, c, h) in enumerate(zip(kinds, cells, hs))])
    meshes = [g.to_solver_mesh() for g in gens]
    mesh_s = time.time() - t0
    # the served stream names no flux or integrator: Rusanov flux and RK2 with
    # multistage limiting for the bump channels.  With the Roe flux the reference's
    # limited scheme has locally unstable modes on some of these channel meshes that
    # grow to a NaN within the 50000-step cap, in plain FP64 as well (--serve-flux
    # roeFlux shows it); the Rusanov flux's dissipation damps them.
    cfgs = [E.load_config(bump_json(float(m), integrator=args.serve_integrator, flux=args.serve_flux) if k == "bump"
                          else cylinder_json(float(r), integrator=args.serve_integrator))
            for k, m, r in zip(kinds, machs, res)]
    L = _lib.load()
    sv = E.EbbServer("split", hbm_budget=int(150e9), build_threads=8)
    clocks = Clocks(0)
    clocks.start()
    tb = time.perf_counter()
    nxt = 0
    ids = {}
    done = {}
    states = {}
    while len(done) < R:
        now = time.perf_counter() - tb
        while nxt < R and arrivals[nxt] <= now:
            ids[sv.submit(meshes[nxt], cfgs[nxt], cap, 1e-8)] = nxt
            nxt += 1
        a, w = sv.tick()
        for r in sv.results():
            k = ids[r["id"]]
            r["latency_s"] = time.perf_counter() - tb - arrivals[k]
            done[k] = r
            if r["status"] == 0:
                states[k] = sv.take_state(r["id"])
        if a == 0:
            time.sleep(0.001)
    wall = time.perf_counter() - tb
    clk = clocks.stop()
    stats = sv.stats()
    sv.close()
    lat = np.array([done[k]["latency_s"] for k in range(R)])
    iters = np.array([done[k]["iterations"] for k in range(R)])
    cu = float(sum(iters[k] * meshes[k].n_cells for k in range(R)))
    # sequential plain FP64: per-step device time alone x steps run
    per = seq_ms_per_step(L, E, meshes, cfgs, "fp64", args.seq_steps, 3)
    seq_s = float(sum(per[k] * iters[k] for k in range(R)) / 1e3)
    # error of the served (split) results against plain FP64 solves with the same stop
    # conditions, on the smallest requests (three bump channels, one cylinder: their
    # FP64 re-solves take seconds)
    err = []
    picks = [k for k in sorted(states, key=lambda k: meshes[k].n_cells) if kinds[k] == "bump"][:3] + \
        [k for k in sorted(states, key=lambda k: meshes[k].n_cells) if kinds[k] == "cyl"][:1]
    for k in picks:
        s64 = E.UfvmSolver(meshes[k], cfgs[k], "fp64")
        s64.set_stop(0, t_end=cfgs[k].t_end, max_steps=cap, resid_drop=1e-8)
        row = {"k": int(k), "kind": str(kinds[k]), "cells": meshes[k].n_cells, "iterations": int(iters[k])}
        try:
            s64.run(10 ** 7, records=False)
            q64, q32 = s64.state, states[k]
            row["fp64_iterations"] = int(s64.status()[0]["iterations"])
            row["l2_rel"] = [float(x) for x in np.sqrt(((q32 - q64) ** 2).mean(axis=0)
                                                       / np.maximum((q64 ** 2).mean(axis=0), 1e-300))]
            row["max_rel"] = float((np.abs(q32 - q64).max(axis=0) / np.maximum(np.abs(q64).max(axis=0), 1e-300)).max())
        except E.EbbError as ex:
            row["fp64_error"] = str(ex)[:120]
        s64.close()
        err.append(row)
    return {"workload": "served-bump70-cyl30-split", "integrator": args.serve_integrator,
            "bump_flux": args.serve_flux, "requests": R,
            "arrival_rate_per_s": 40.0,
            "cells_range": [int(cells.min()), int(cells.max())], "cells_total": int(sum(m.n_cells for m in meshes)),
            "step_cap": cap, "resid_drop": 1e-8, "wall_s": wall, "solves_per_s": R / wall,
            "cell_updates_per_s": cu / wall, "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)), "latency_max_s": float(lat.max()),
            "statuses": sorted(set(int(done[k]["status"]) for k in range(R))),
            "failed": [{"k": k, "kind": str(kinds[k]), "cells": meshes[k].n_cells, "status": int(done[k]["status"]),
                        "iterations": int(done[k]["iterations"])} for k in range(R) if done[k]["status"] != 0],
            "done_reasons": {str(v): int((np.array([done[k]["done_reason"] for k in range(R)]) == v).sum())
                             for v in (0, 1, 2, 3)},
            "sequential_fp64": {"est_total_s": seq_s, "cell_updates_per_s": cu / seq_s,
                                "sample": "%d timed steps per request alone after 3 warm-up, x steps run"
                                          % args.seq_steps},
            "throughput_vs_sequential_fp64": (cu / wall) / (cu / seq_s), "bytes_peak": stats["bytes_peak"],
            "error_vs_fp64": err, "mesh_s": round(mesh_s, 1), "clocks": clk}


def run_reference(args, ws, rank):
    from ebbcfd_gb300 import meshgen
    from oracle import gmsh_ref, ref
    gen = meshgen.wedge(args.cells, seed=0)
    nthreads = ref.max_threads()
    ref.set_threads(nthreads)
    om = ref.OracleMesh(gen.as_reader_dict(), gmsh_ref.load_config(wedge_config()))
    ncell = om.n_cells
    om.run(args.warmup)
    t0 = time.perf_counter()
    om.run(1)
    t1 = time.perf_counter() - t0
    n = int(max(1, min(args.steps, args.cpu_budget * 4 / max(t1, 1e-6))))
    t0 = time.perf_counter()
    if n > 1:
        om.run(n - 1)
    t = time.perf_counter() - t0 + t1
    v = ncell * n / t
    return {"impl": "reference", "metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": ws,
            "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * t / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "wedge-M2.5-rusanov-rk2-cfl0.4", "cells": ncell, "precision": "plain-fp64"},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": nthreads, "kind": "port",
                             "sample": "%d of %d requested RK2 steps of the full %d-cell wedge" % (n, args.steps,
                                                                                                   ncell)},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=1_000_000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-split", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--workload", default="wedge",
                    choices=["wedge", "wedge5000", "mms32", "plate4m", "batch512", "serve"])
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--seq-stride", type=int, default=4)
    ap.add_argument("--seq-steps", type=int, default=100)
    ap.add_argument("--requests", type=int, default=32)
    ap.add_argument("--max-cells", type=float, default=2e6)
    ap.add_argument("--step-cap", type=int, default=50000)
    ap.add_argument("--serve-integrator", default="RK2", choices=["Euler", "RK2", "RK2_TVD", "RK4"])
    ap.add_argument("--serve-flux", default="rusanovFlux", choices=["roeFlux", "rusanovFlux"])
    ap.add_argument("--batch-precision", default="split", choices=["split", "fp64"])
    args = ap.parse_args()
    args.steps_given = "--steps" in sys.argv
    args.cells_given = "--cells" in sys.argv
    args.warmup = max(3, args.warmup)
    ws, rank, local = dist_env()
    if args.workload != "wedge":
        # accuracy/throughput reports for the other configurations (not the headline line)
        run = {"mms32": run_mms32, "plate4m": run_plate, "batch512": run_batch512, "serve": run_serve,
               "wedge5000": run_wedge5000}
        out = run[args.workload](args)
        print(json.dumps(out))
        return
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, ws, rank)))
        return
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    out = run_ours(args, ws, rank, local)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
