#!/usr/bin/env python3
"""Throughput of the explicit unstructured FV update on GB300.

Workload (default): the laminar Navier-Stokes flat plate -- domain [-0.5,2]x[0,0.5],
4.0M mixed cells (anisotropic wall-layer quads, first-cell height 1e-4, growth 1.05;
seeded-Delaunay triangles above), Mach 0.3, Re_L 1e5, Pr 0.72, adiabatic no-slip wall
for x >= 0, Roe + viscous flux, limited second order, RK4 at CFL 0.8.  A step is one
RK4 time step of the whole mesh (four residual evaluations with their stage updates,
then the per-step reductions of the time loop); the metric is cell-updates/s = cells
x steps / time.  `value` is the plain FP64 path (the reference's own precision and
operation order); `split_path` beside it is the FP32/FP64 split precision form from
the same initial state, with its speed-up and its error against FP64 for drag, lift,
the wall skin friction, the residual history and the state.  The ~4M-cell working set
(~2.4 GB FP64) exceeds the 129 MB L2, so no flush is needed between steps.  `wedge`
repeats the measurement on the 1.0M-cell Mach 2.5 wedge (Rusanov, RK2, CFL 0.4).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference-semantics FP64 CPU restatement (oracle/) on all
host cores on the same plate mesh and config (the D reference cannot be built: no D
compiler, MPI or ParMETIS is installed).  N>1: one independent replica per GPU (the
path does not shard), weak scaling.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WEDGE_BCS = [{"tag": "Inflow", "type": "fullState", "q": [2.5, 0, 1, 1]},
             {"tag": "Top", "type": "fullState", "q": [2.5, 0, 1, 1]},
             {"tag": "Symmetry", "type": "symmetry", "q": [2.5, 0, 1, 1]},
             {"tag": "Ramp", "type": "inviscidWall", "q": [2.5, 0, 1, 1]},
             {"tag": "Outflow", "type": "fullState", "q": [2.5, 0, 1, 1]}]

PLATE_WORKLOAD = "ns-plate-M0.3-Re1e5-roe-visc-rk4-cfl0.8"
WEDGE_WORKLOAD = "wedge-M2.5-rusanov-rk2-cfl0.4"


def wedge_config(cfl=0.4):
    return json.dumps({"mesh": "wedge.msh", "dt": 1e-4, "tEnd": 1e9, "flux": "rusanovFlux", "saveIter": -1,
                       "plotIter": -1, "forceBoundary": "Ramp", "integrator": "RK2", "limited": True, "CFL": cfl,
                       "initialConditions": [2.5, 0, 1, 1], "boudaryConditions": WEDGE_BCS})


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


# what each headline workload runs: mesh generator, config, force tag, stages per step
WORKLOADS = {
    "plate": {"name": PLATE_WORKLOAD, "cells": 4_000_000, "config": plate_config, "force_tag": "Wall",
              "stages": 4, "need_grad": True, "integrator": "RK4"},
    "wedge": {"name": WEDGE_WORKLOAD, "cells": 1_000_000, "config": wedge_config, "force_tag": "Ramp",
              "stages": 2, "need_grad": False, "integrator": "RK2"},
}


def make_mesh(kind, cells):
    from ebbcfd_gb300 import meshgen
    return meshgen.flat_plate(cells) if kind == "plate" else meshgen.wedge(cells, seed=0)


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
    """SM clock, its maximum, power and the active clock-event reasons of the GPU,
    sampled every 2 ms by a host thread during the timed region through NVML's
    read-only queries (libnvidia-ml, loaded with ctypes); nvidia-smi at 50 ms when NVML
    cannot be loaded.  The timed calls release the interpreter lock (ctypes), so the
    thread samples while the GPU works."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    REASONS = {0x2: "applications_clocks_setting", 0x4: "sw_power_cap", 0x8: "hw_slowdown",
               0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.src = None
        self._stop = threading.Event()
        self._t = None
        self.p = None

    def _nvml_handle(self):
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            return None, None
        h = ctypes.c_void_p()
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")
        sel = vis[self.device].strip() if vis and vis[0] != "" and self.device < len(vis) else str(self.device)
        if sel.startswith("GPU-") or sel.startswith("MIG-"):
            r = nv.nvmlDeviceGetHandleByUUID(sel.encode(), ctypes.byref(h))
        else:
            r = nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(int(sel)), ctypes.byref(h))
        return (nv, h) if r == 0 else (None, None)

    def _run_nvml(self, nv, h):
        sm, mx, pw, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self._stop.is_set():
            if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm)) == 0 and \
                    nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
                ok_r = reasons(h, ctypes.byref(rs)) == 0
                ok_p = nv.nvmlDeviceGetPowerUsage(h, ctypes.byref(pw)) == 0
                self.rows.append((float(sm.value), float(mx.value), pw.value / 1e3 if ok_p else None,
                                  int(rs.value) if ok_r else 0))
            time.sleep(0.002)

    def start(self):
        try:
            nv, h = self._nvml_handle()
        except OSError:
            nv, h = None, None
        if nv is not None:
            self.src = "nvml, 2 ms"
            self._t = threading.Thread(target=self._run_nvml, args=(nv, h), daemon=True)
            self._t.start()
            return
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
            self.src = "nvidia-smi, 50 ms"
        except Exception:
            self.p = None

    def stop(self):
        if self._t is not None:
            self._stop.set()
            self._t.join()
        elif self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.flush()
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            bits = [0x8, 0x40, 0x20, 0x4]
            for line in open(self.f.name):
                r = [x.strip() for x in line.split(",")]
                if len(r) >= 9 and r[1].replace(".", "").isdigit() and r[2].replace(".", "").isdigit():
                    rs = sum(b for b, k in zip(bits, range(4)) if r[5 + k] == "Active")
                    pw = float(r[3]) if r[3].replace(".", "").isdigit() else None
                    self.rows.append((float(r[1]), float(r[2]), pw, rs))
            os.unlink(self.f.name)
        if not self.rows:
            return None
        sm = [r[0] for r in self.rows]
        pw = [r[2] for r in self.rows if r[2] is not None]
        reasons = sorted({n for r in self.rows for b, n in self.REASONS.items() if r[3] & b})
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": max(r[1] for r in self.rows),
                "reasons": reasons, "samples": len(self.rows), "power_w_max": max(pw) if pw else None,
                "source": self.src}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_counters(kernel, precision, workload, ncell):
    """DRAM bytes (read + write) per launch of `kernel` and its FP64- and FMA-pipe
    shares from the committed ncu summaries under profiles/: lines "traffic: <kernel>
    <precision> <bytes> <workload> <cells>", "fp64pipe: <kernel> <precision> <percent>
    <workload>" and "fmapipe: ..." alike (a capture of `cells` cells of the workload;
    traffic is scaled to `ncell` cells: it grows with the cells processed).  None when
    no capture covers the kernel."""
    import glob
    import re
    out = {"traffic": None, "fp64_pipe_pct": None, "fma_pipe_pct": None}
    for f in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        for line in open(f):
            m = re.match(r"traffic: (\S+) (\S+) (\d+) (\S+) (\d+)\s*$", line)
            if m and m.group(1) == kernel and m.group(2) == precision and m.group(4) == workload:
                cells = int(m.group(5))
                out["traffic"] = {"bytes": int(m.group(3)) * ncell / cells, "source": os.path.relpath(f, ROOT),
                                  "captured_cells": cells}
            m = re.match(r"(fp64|fma)pipe: (\S+) (\S+) ([\d.]+) (\S+)\s*$", line)
            if m and m.group(2) == kernel and m.group(3) == precision and m.group(5) == workload:
                out[m.group(1) + "_pipe_pct"] = float(m.group(4))
    return out


def algorithmic_bytes(info, real=8, need_grad=False, limited=True):
    """Bytes each kernel must move per launch, every array touched once (re-reads of
    a neighbour's state count 0).  S = face slots, E = interior edges, G = boundary
    edges; real = bytes of the arithmetic type (8 plain FP64, 4 split).  need_grad:
    viscous terms, k_cell writes each cell's gradient and k_flux reads it (with the
    edge's two cell ids).  The update figure is a first RK stage (the stage
    ebb_profile_kernels times)."""
    C, S, E, G = info.n_cells, info.face_slots, info.n_int_edges, info.n_ghost
    r = real
    cell = C * (4 * r + 4) + S * (4 + 2 * r + (2 * r if limited else 0) + 2 * r) + S * 4 * r + (C * 8 * r if need_grad else 0)
    flux = E * (8 + 2 * r + r + 8 * r + 5 * r) + G * (12 + 2 * r + r + 4 * r + 4 * r + 5 * r)
    if need_grad:
        flux += E * 8 + (C + G) * 8 * r
    # residual + first-stage update: nedge, perim, d, -1/area, FP64 q read, aux write
    # (T) and next-stage state write (T)
    update = C * (4 + 3 * r + 32 + 4 * r + 4 * r) + S * 4 + (E + G) * 5 * r
    if r == 4:  # split: the freestream correction reads the stage state and each slot's normal and length
        update += C * 4 * r + S * 3 * r
    return {"cell": cell, "flux": flux, "update": update}


def wall_cf(edges, efl, tag_index):
    """Skin friction of a viscous wall per wall edge: the wall shear is the x-momentum
    flux F1 = len*F1 / len of each wall edge (the wall is y = 0, n = (0, -1), so
    F1 = -Fv1 = mu du/dy), and Cf = shear / (0.5 rho U^2) with the freestream rho = U = 1.
    Returns (x of the edge midpoints, Cf), sorted by x."""
    m = edges["group"] == tag_index
    x = edges["mid"][m, 0]
    cf = 2.0 * efl[m, 1] / edges["len"][m]
    o = np.argsort(x)
    return x[o], cf[o]


def rel_l2(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b ** 2), 1e-300)))


def measure(L, E, _lib, mesh, wl, precision, args, local, ws, want_e2e, hist_steps):
    """One precision form on one workload: `hist_steps` recorded steps (warm-up, and
    the force and residual history), per-kernel event times, `args.steps` timed steps
    (CUDA events on the solver stream, inputs resident), then the end-to-end run
    through the C ABI with host copies every step."""
    import ctypes as C
    cfg = E.load_config(wl["config"]())
    t0 = time.time()
    sol = E.UfvmSolver(mesh, cfg, precision=precision)
    setup_s = time.time() - t0
    info = mesh.info
    ncell = info.n_cells
    hist = sol.run(max(args.warmup, hist_steps), records=True)
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
    st = sol.status()[0]
    efl = sol.edge_fluxes()
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
    ab = algorithmic_bytes(info, real=4 if precision == "split" else 8, need_grad=wl["need_grad"])
    kernels = {}
    for k in ("cell", "flux", "update"):
        sec = kern_ms[k] * 1e-3
        cnt = profiled_counters("k_" + k, precision, wl["name"], ncell)
        row = {"ms": kern_ms[k], "algorithmic_bytes": ab[k], "achieved_gbs": ab[k] / sec / 1e9,
               "frac": ab[k] / sec / 1e9 / peak}
        if cnt["traffic"]:
            row["dram_bytes"] = cnt["traffic"]["bytes"]
            row["dram_gbs"] = cnt["traffic"]["bytes"] / sec / 1e9
            row["frac_dram"] = row["dram_gbs"] / peak
            row["traffic_source"] = cnt["traffic"]
        for pipe in ("fp64", "fma"):
            if cnt[pipe + "_pipe_pct"] is not None:
                row[pipe + "_pipe_active_pct"] = cnt[pipe + "_pipe_pct"]
        kernels["k_" + k] = row
    dom = max(("cell", "flux", "update"), key=lambda k: kern_ms[k])
    d = kernels["k_" + dom]
    roof = {"bound": "hbm", "kernel": "k_" + dom, "achieved": d["achieved_gbs"], "peak": peak, "unit": "GB/s",
            "frac": d["frac"], "achieved_basis": "algorithmic bytes per launch (model) / event-timed launch",
            "frac_dram": d.get("frac_dram"), "peak_source": peak_kind, "traffic": d.get("dram_bytes"),
            "kernels": kernels, "step_end_ms": kern_ms["step_end"]}
    if precision == "fp64":
        roof["limiter"] = "FP64 pipe (ncu fp64_pipe_active_pct; GB300 runs FP64 at a small fraction of FP32)"
    elif precision == "df":
        roof["limiter"] = ("FP32 (FMA) pipe and instruction issue: double-float arithmetic takes 5-20 FP32 "
                           "instructions per operation (ncu fma_pipe_active_pct)")
    sol.close()
    return {"value": value, "elapsed": elapsed, "steps": steps_done, "setup_s": setup_s, "roofline": roof,
            "e2e": e2e, "clocks": clk, "state": state, "hist": hist, "status": st, "edge_fluxes": efl}


def split_errors(mesh, wl, m64, m32):
    """Error of the split precision form against plain FP64 from the same initial state
    after the same steps: drag and lift, the force tag's wall shear (Cf per wall edge,
    viscous walls), the recorded residual and force history, and the state."""
    q64, q32 = m64["state"], m32["state"]
    scale = np.maximum(np.abs(q64).max(axis=0), 1e-300)
    h64, h32 = m64["hist"], m32["hist"]
    nh = min(len(h64), len(h32))
    r64, r32 = h64[:nh, 3:7], h32[:nh, 3:7]
    rel_r = np.abs(r32 / np.where(r64 == 0, 1e-300, r64) - 1)
    d64, d32 = h64[:nh, 1], h32[:nh, 1]
    out = {"steps_compared": int(m64["steps"] + nh),
           "drag": [m64["status"]["drag"], m32["status"]["drag"]],
           "drag_rel_err": abs(m32["status"]["drag"] / m64["status"]["drag"] - 1),
           "lift": [m64["status"]["lift"], m32["status"]["lift"]],
           "lift_abs_err_over_drag": abs(m32["status"]["lift"] - m64["status"]["lift"]) / abs(m64["status"]["drag"]),
           "history_steps": int(nh),
           "resid_history_rel_err_max": float(rel_r.max()), "resid_history_rel_err_median": float(np.median(rel_r)),
           "drag_history_rel_err_max": float(np.max(np.abs(d32 / d64 - 1))),
           "state_l2_err_vs_fp64": [float(x) for x in np.sqrt(((q32 - q64) ** 2).mean(axis=0)
                                                               / np.maximum((q64 ** 2).mean(axis=0), 1e-300))],
           "state_max_err_vs_fp64": float((np.abs(q32 - q64).max(axis=0) / scale).max())}
    if wl["need_grad"]:
        edges = mesh.edges()
        ti = mesh.tags.index(wl["force_tag"])
        x, cf64 = wall_cf(edges, m64["edge_fluxes"], ti)
        _, cf32 = wall_cf(edges, m32["edge_fluxes"], ti)
        out["cf_rel_l2_err"] = rel_l2(cf32, cf64)
        out["cf_max_err_over_max_cf"] = float(np.abs(cf32 - cf64).max() / max(np.abs(cf64).max(), 1e-300))
        out["wall_edges"] = int(len(x))
    return out


def run_workload(kind, args, ws, rank, local, want_cpu, cells=None):
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib

    wl = WORKLOADS[kind]
    L = _lib.load()
    L.ebb_set_device(local)
    t0 = time.time()
    gen = make_mesh(kind, cells or wl["cells"])
    mesh = gen.to_solver_mesh()
    mesh_s = time.time() - t0
    info = mesh.info
    ncell = info.n_cells
    hist_steps = args.hist_steps
    m64 = measure(L, E, _lib, mesh, wl, "fp64", args, local, ws, not args.no_e2e, hist_steps)
    split = None
    if not args.no_split:
        m32 = measure(L, E, _lib, mesh, wl, "split", args, local, ws, not args.no_e2e, hist_steps)
        split = {"value": m32["value"], "unit": "cell-updates/s", "ms_per_step": 1e3 * m32["elapsed"] / m32["steps"],
                 "speedup_vs_fp64": m32["value"] / m64["value"], "roofline": m32["roofline"],
                 "error_vs_fp64": split_errors(mesh, wl, m64, m32), "clocks": m32["clocks"], "e2e": m32["e2e"]}
    dfl = None
    if not args.no_df:
        mdf = measure(L, E, _lib, mesh, wl, "df", args, local, ws, not args.no_e2e, hist_steps)
        dfl = {"value": mdf["value"], "unit": "cell-updates/s", "ms_per_step": 1e3 * mdf["elapsed"] / mdf["steps"],
               "speedup_vs_fp64": mdf["value"] / m64["value"], "roofline": mdf["roofline"],
               "error_vs_fp64": split_errors(mesh, wl, m64, mdf), "clocks": mdf["clocks"], "e2e": mdf["e2e"]}
    cpu = None
    if rank == 0 and want_cpu:
        cpu = cpu_baseline(gen, kind, ncell, budget_s=args.cpu_budget)
    steps_done = m64["steps"]
    stages = wl["stages"]
    return {
        "metric": "cell-updates/s", "value": m64["value"], "unit": "cell-updates/s", "n_gpus": ws,
        "steps": steps_done, "warmup": max(args.warmup, hist_steps), "ms_per_step": 1e3 * m64["elapsed"] / max(1, steps_done),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl["name"], "cells": ncell, "faces": info.face_slots,
                   "interior_edges": info.n_int_edges, "boundary_edges": info.n_ghost, "precision": "plain-fp64",
                   "integrator": wl["integrator"],
                   "l2": "inputs larger than L2 (~%d MB resident)" % (sol_bytes(info, wl["need_grad"]) // 2 ** 20),
                   "parallelism": "replicas" if ws > 1 else "single", "mesh_s": round(mesh_s, 2),
                   "setup_s": round(m64["setup_s"], 2)},
        "cell_stages_per_s": stages * m64["value"], "roofline": m64["roofline"], "cpu_baseline": cpu,
        "e2e": m64["e2e"], "gpu_launches": steps_done * (3 * stages + 1), "clocks": m64["clocks"],
        "split_path": split, "df_path": dfl,
    }


def sol_bytes(info, need_grad=False):
    C, S, E, G = info.n_cells, info.face_slots, info.n_int_edges, info.n_ghost
    return 8 * (12 * (C + G) + 4 * 4 * S // 3 + 8 * (C + G) + 5 * (E + G) + 12 * S)


def cpu_baseline(gen, kind, ncell, budget_s=20.0, steps_max=1000):
    from oracle import gmsh_ref, ref
    wl = WORKLOADS[kind]
    nthreads = ref.max_threads()
    ref.set_threads(nthreads)
    om = ref.OracleMesh(gen.as_reader_dict(), gmsh_ref.load_config(wl["config"]()))
    t0 = time.perf_counter()
    om.run(1)
    t1 = time.perf_counter() - t0
    n = int(max(1, min(steps_max, budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    om.run(n)
    t = time.perf_counter() - t0
    ref.set_threads(1)
    return {"value": ncell * n / t, "unit": "cell-updates/s", "cores": nthreads, "kind": "port",
            "sample": "%d %s steps of the full %d-cell %s (after 1 untimed step)" % (n, wl["integrator"], ncell,
                                                                                     wl["name"])}


def mms32_config():
    return json.dumps({"mesh": "quads32.msh", "dt": 1e-4, "tEnd": 1e9, "flux": "roeFlux", "saveIter": -1,
                       "plotIter": -1, "forceBoundary": "Freestream", "integrator": "RK2_TVD", "limited": True,
                       "CFL": 0.5, "cflAdjust": False, "initialConditions": [0.5, 0, 1, 1],
                       "boudaryConditions": [{"tag": "Freestream", "type": "dirichlet", "q": [0.5, 0, 1, 1]}]})


def run_mms32(args):
    """32x32 quads on [0,1]^2, the sine manufactured fields, Dirichlet boundaries, Roe,
    limited, TVD-RK2, CFL 0.5, 1000 steps: L2(rho) error vs the exact field for the
    oracle, the plain FP64 path (which must equal it bitwise), the split path and the
    double-float path."""
    import ctypes as C
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib, meshgen
    from oracle import gmsh_ref, ref
    L = _lib.load()
    gen = meshgen.uniform_quads(32)
    steps = args.steps if args.steps_given else 1000
    out = {"workload": "mms32-sine-roe-tvd-cfl0.5", "cells": 1024, "steps": steps}
    q_exact, _, _ = ref.mms_eval(2, gen.to_solver_mesh().centroids())
    for prec in ("fp64", "split", "df"):
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
    for prec in ("split", "df"):
        out[prec + "_l2_rel_diff"] = abs(out[prec]["l2_rho"] / out["fp64"]["l2_rho"] - 1)
        out[prec + "_state_max_rel_err"] = float((np.abs(out[prec]["state"] - qo).max(axis=0)
                                                  / np.abs(qo).max(axis=0)).max())
    for prec in ("fp64", "split", "df"):
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
    """Accuracy of the wedge run: the 1M-cell Mach 2.5 wedge run 5000 RK2 steps in
    plain FP64 (bitwise equal to the oracle on the parity cases, and used here as the
    reference solution: the oracle would take ~7 min on the host), in split precision
    and in double-float; shock angle of each against the oblique-shock relation, and
    the split and double-float paths' state, drag and lift errors against FP64 (forces
    on the ramp)."""
    import ctypes as C
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib, meshgen
    L = _lib.load()
    steps = args.steps if args.steps_given else 5000
    mesh = meshgen.wedge(args.cells if args.cells_given else WORKLOADS["wedge"]["cells"], seed=0).to_solver_mesh()
    xy = mesh.centroids()
    out = {"workload": "wedge-M2.5-rusanov-rk2-cfl0.4-accuracy", "cells": mesh.n_cells, "steps": steps,
           "theory_shock_angle_deg": theory_shock_angle()}
    qs, forces = {}, {}
    for prec in ("fp64", "split", "df"):
        s = E.UfvmSolver(mesh, E.load_config(wedge_config()), precision=prec)
        n = C.c_int64()
        ms = C.c_double()
        code = L.ebb_run_timed(s.h, steps, C.byref(n), C.byref(ms))
        if code:
            s._raise(code)
        q = s.state
        qs[prec] = q
        st = s.status()[0]
        forces[prec] = (st["drag"], st["lift"])
        t_end = s.time()[0]
        # the corner shock is established within about the distance the flow has moved
        span = min(1.1, 0.9 * t_end)
        beta, x0 = shock_angle(xy, q, x_lo=0.5 + 0.15 * span, x_hi=0.5 + 0.85 * span, nbins=10)
        out[prec] = {"cell_updates_per_s": mesh.n_cells * n.value / (ms.value / 1e3), "shock_angle_deg": beta,
                     "shock_origin_x": x0, "t": t_end, "shock_window_x": [0.5 + 0.15 * span, 0.5 + 0.85 * span],
                     "drag": st["drag"], "lift": st["lift"]}
        s.close()
    d64, l64 = forces["fp64"]
    for prec in ("split", "df"):
        d = qs[prec] - qs["fp64"]
        out[prec + "_l2_rel_err"] = [float(np.sqrt(np.mean(d[:, k] ** 2)) / np.sqrt(np.mean(qs["fp64"][:, k] ** 2)))
                                     for k in range(4)]
        out[prec + "_max_rel_err"] = float((np.abs(d).max(axis=0) / np.abs(qs["fp64"]).max(axis=0)).max())
        out[prec + "_drag_rel_err"] = abs(forces[prec][0] - d64) / abs(d64)
        out[prec + "_lift_rel_err"] = abs(forces[prec][1] - l64) / abs(l64)
    return out


def run_plate20k(args):
    """The Navier-Stokes plate run to its end: the 4.0M-cell plate (RK4, CFL 0.8),
    20000 steps in plain FP64 and in split precision from the same initial state, every
    step's drag and residuals recorded.  Reports each path's throughput, the drag
    coefficient Cd = drag / (0.5 rho U^2 L_w) (wall length L_w = 2, x in [0, 2]), the
    wall skin friction Cf(x) per x band, the split path's error against FP64 for each,
    and the Blasius laminar value 0.664 / sqrt(Re_x) beside Cf (the boundary layer forms
    from the leading edge; at time t it has developed over roughly x < t)."""
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib
    _lib.load()
    steps = args.steps if args.steps_given else 20000
    t0 = time.time()
    gen = make_mesh("plate", args.cells if args.cells_given else 4_000_000)
    mesh = gen.to_solver_mesh()
    mesh_s = time.time() - t0
    edges = mesh.edges()
    ti = mesh.tags.index("Wall")
    out = {"workload": PLATE_WORKLOAD + "-full", "cells": mesh.n_cells, "steps": steps, "mesh_s": round(mesh_s, 1)}
    res = {}
    for prec in ("fp64", "split", "df"):
        sol = E.UfvmSolver(mesh, E.load_config(plate_config()), precision=prec)
        clocks = Clocks(0)
        clocks.start()
        t1 = time.perf_counter()
        err = None
        try:
            rec = sol.run(steps, records=True)
        except E.EbbError as ex:
            err = str(ex)[:160]
            rec = None
        wall = time.perf_counter() - t1
        clk = clocks.stop()
        t_end, dt_end, it = sol.time()
        row = {"iterations": int(it), "t": t_end, "dt": dt_end, "wall_s": wall,
               "cell_updates_per_s": mesh.n_cells * it / wall, "clocks": clk}
        if err:
            row["error"] = err
        else:
            x, cf = wall_cf(edges, sol.edge_fluxes(), ti)
            row["drag"] = float(rec[-1, 1])
            row["cd"] = float(rec[-1, 1] / (0.5 * 2.0))
            row["lift"] = float(rec[-1, 2])
            row["resid_last"] = [float(v) for v in rec[-1, 3:7]]
            res[prec] = {"rec": rec, "x": x, "cf": cf, "state": sol.state}
        out[prec] = row
        sol.close()
    if "fp64" in res and "split" in res:
        a, b = res["fp64"], res["split"]
        n = min(len(a["rec"]), len(b["rec"]))
        d64, d32 = a["rec"][:n, 1], b["rec"][:n, 1]
        r64, r32 = a["rec"][:n, 3:7], b["rec"][:n, 3:7]
        out["split_drag_rel_err"] = abs(b["rec"][n - 1, 1] / a["rec"][n - 1, 1] - 1)
        out["split_cd_abs_err"] = abs(b["rec"][n - 1, 1] - a["rec"][n - 1, 1]) / (0.5 * 2.0)
        out["split_drag_history_rel_err_max"] = float(np.max(np.abs(d32 / d64 - 1)))
        rr = np.abs(r32 / np.where(r64 == 0, 1e-300, r64) - 1)
        out["split_resid_history_rel_err"] = {"max": float(rr.max()), "median": float(np.median(rr)),
                                              "at_steps": {str(k): float(rr[k - 1].max()) for k in
                                                           (1, 10, 100, 1000, 5000, 10000, 20000) if k <= n}}
        out["split_cf_rel_l2_err"] = rel_l2(b["cf"], a["cf"])
        out["split_cf_max_err_over_max_cf"] = float(np.abs(b["cf"] - a["cf"]).max() / np.abs(a["cf"]).max())
        q64, q32 = a["state"], b["state"]
        out["split_state_l2_err"] = [float(v) for v in np.sqrt(((q32 - q64) ** 2).mean(axis=0)
                                                               / np.maximum((q64 ** 2).mean(axis=0), 1e-300))]
        out["split_speedup"] = out["split"]["cell_updates_per_s"] / out["fp64"]["cell_updates_per_s"]
        bands = [0.0, 0.02, 0.05, 0.1, 0.2, 0.3, 0.5, 1.0, 1.5, 2.0]
        table = []
        x = a["x"]
        for lo, hi in zip(bands[:-1], bands[1:]):
            m = (x >= lo) & (x < hi)
            if not m.any():
                continue
            xc = float(x[m].mean())
            table.append({"x_band": [lo, hi], "edges": int(m.sum()), "cf_fp64": float(a["cf"][m].mean()),
                          "cf_split": float(b["cf"][m].mean()),
                          "cf_rel_err": float(abs(b["cf"][m].mean() / a["cf"][m].mean() - 1)),
                          "cf_blasius_at_mean_x": 0.664 / np.sqrt(1e5 * xc) if xc > 0 else None})
        out["cf_table"] = table
    if "fp64" in res and "df" in res:
        a, w = res["fp64"], res["df"]
        n = min(len(a["rec"]), len(w["rec"]))
        rr = np.abs(w["rec"][:n, 3:7] / np.where(a["rec"][:n, 3:7] == 0, 1e-300, a["rec"][:n, 3:7]) - 1)
        out["df_speedup"] = out["df"]["cell_updates_per_s"] / out["fp64"]["cell_updates_per_s"]
        out["df_drag_rel_err"] = abs(w["rec"][n - 1, 1] / a["rec"][n - 1, 1] - 1)
        out["df_drag_history_rel_err_max"] = float(np.max(np.abs(w["rec"][:n, 1] / a["rec"][:n, 1] - 1)))
        out["df_cf_rel_l2_err"] = rel_l2(w["cf"], a["cf"])
        out["df_resid_history_rel_err"] = {"max": float(rr.max()), "median": float(np.median(rr))}
        out["df_state_l2_err"] = [float(v) for v in np.sqrt(((w["state"] - a["state"]) ** 2).mean(axis=0)
                                                            / np.maximum((a["state"] ** 2).mean(axis=0), 1e-300))]
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
    split precision, continued in plain FP64 (--finish df: double-float) once its
    residual levels off (the server's finishing); admission capped at 150 GB.  Latency =
    result in hand minus scheduled arrival; service time = finish minus first admission.
    The sequential baselines solve the requests one at a time: each request's device
    time per step alone (timed on a sample of steps) times the steps it ran -- all in
    plain FP64, or in the served form (its split steps in split precision, the rest in
    the finishing form)."""
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
    sv = E.EbbServer("split", hbm_budget=int(150e9), build_threads=8, finish_fp64=int(not args.no_finish),
                     finish_precision=args.finish)
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
    svc = np.array([done[k]["finish_s"] - done[k]["admit_s"] for k in range(R)])
    iters = np.array([done[k]["iterations"] for k in range(R)])
    it32 = np.array([min(done[k]["split_iterations"], done[k]["iterations"]) for k in range(R)])
    cu = float(sum(iters[k] * meshes[k].n_cells for k in range(R)))
    # sequential solves: per-step device time alone x steps run (plain FP64 throughout,
    # or split steps in split precision and the finishing steps in the finishing form)
    per = seq_ms_per_step(L, E, meshes, cfgs, "fp64", args.seq_steps, 3)
    per32 = seq_ms_per_step(L, E, meshes, cfgs, "split", args.seq_steps, 3)
    perF = per if args.finish == "fp64" else seq_ms_per_step(L, E, meshes, cfgs, args.finish, args.seq_steps, 3)
    seq_s = float(sum(per[k] * iters[k] for k in range(R)) / 1e3)
    seq32_s = float(sum(per32[k] * it32[k] + perF[k] * (iters[k] - it32[k]) for k in range(R)) / 1e3)
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
            "service_p50_s": float(np.percentile(svc, 50)), "service_p99_s": float(np.percentile(svc, 99)),
            "finish_precision": args.finish,
            "finished_after_stall": int(sum(done[k]["escalated"] == 2 for k in range(R))),
            "split_iteration_share": float(sum(it32[k] * meshes[k].n_cells for k in range(R)) / cu),
            "statuses": sorted(set(int(done[k]["status"]) for k in range(R))),
            "failed": [{"k": k, "kind": str(kinds[k]), "cells": meshes[k].n_cells, "status": int(done[k]["status"]),
                        "iterations": int(done[k]["iterations"])} for k in range(R) if done[k]["status"] != 0],
            "done_reasons": {str(v): int((np.array([done[k]["done_reason"] for k in range(R)]) == v).sum())
                             for v in (0, 1, 2, 3)},
            "sequential_fp64": {"est_total_s": seq_s, "cell_updates_per_s": cu / seq_s,
                                "sample": "%d timed steps per request alone after 3 warm-up, x steps run"
                                          % args.seq_steps},
            "sequential_served_form": {"est_total_s": seq32_s, "cell_updates_per_s": cu / seq32_s,
                                       "sample": "split steps at the split path's time per step alone, the rest at "
                                                 "the %s form's" % args.finish},
            "throughput_vs_sequential_fp64": (cu / wall) / (cu / seq_s),
            "throughput_vs_sequential_served_form": (cu / wall) / (cu / seq32_s), "bytes_peak": stats["bytes_peak"],
            "error_vs_fp64": err, "mesh_s": round(mesh_s, 1), "clocks": clk}


def run_reference(args, ws, rank):
    """The reference-semantics FP64 CPU restatement (oracle/, OpenMP over all host
    threads) on the headline workload: the same mesh generator, config, metric and
    unit; steps bounded so that the whole run stays within a few minutes."""
    from oracle import gmsh_ref, ref
    kind = args.workload
    wl = WORKLOADS[kind]
    gen = make_mesh(kind, args.cells if args.cells_given else wl["cells"])
    nthreads = ref.max_threads()
    ref.set_threads(nthreads)
    om = ref.OracleMesh(gen.as_reader_dict(), gmsh_ref.load_config(wl["config"]()))
    ncell = om.n_cells
    t0 = time.perf_counter()
    om.run(1)
    t1 = time.perf_counter() - t0
    # warm-up (at most the budget allows), then a bounded number of timed steps
    nw = int(max(0, min(args.warmup - 1, args.cpu_budget / max(t1, 1e-6))))
    if nw:
        om.run(nw)
    n = int(max(1, min(args.steps, args.cpu_budget * 4 / max(t1, 1e-6))))
    t0 = time.perf_counter()
    om.run(n)
    t = time.perf_counter() - t0
    v = ncell * n / t
    return {"impl": "reference", "metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": ws,
            "steps": n, "warmup": nw + 1, "ms_per_step": 1e3 * t / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["name"], "cells": ncell, "precision": "plain-fp64",
                       "integrator": wl["integrator"]},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": nthreads, "kind": "port",
                             "sample": "%d of %d requested %s steps of the full %d-cell %s" % (
                                 n, args.steps, wl["integrator"], ncell, wl["name"])},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=None, help="cells of the headline mesh")
    ap.add_argument("--wedge-cells", type=int, default=1_000_000)
    ap.add_argument("--hist-steps", type=int, default=100,
                    help="recorded steps before the timed ones (warm-up and the split path's history error)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-split", action="store_true")
    ap.add_argument("--finish", default="fp64", choices=["fp64", "df"],
                    help="serve: form a stalled split solve finishes in")
    ap.add_argument("--no-wedge", action="store_true")
    ap.add_argument("--no-df", action="store_true", help="skip the double-float precision form's leg")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--workload", default="plate",
                    choices=["plate", "wedge", "plate20k", "wedge5000", "mms32", "batch512", "serve"])
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--seq-stride", type=int, default=4)
    ap.add_argument("--seq-steps", type=int, default=100)
    ap.add_argument("--requests", type=int, default=32)
    ap.add_argument("--max-cells", type=float, default=2e6)
    ap.add_argument("--step-cap", type=int, default=50000)
    ap.add_argument("--serve-integrator", default="RK2", choices=["Euler", "RK2", "RK2_TVD", "RK4"])
    ap.add_argument("--serve-flux", default="rusanovFlux", choices=["roeFlux", "rusanovFlux"])
    ap.add_argument("--batch-precision", default="split", choices=["split", "fp64"])
    ap.add_argument("--no-finish", action="store_true", help="served split solves without finishing")
    args = ap.parse_args()
    args.steps_given = "--steps" in sys.argv
    args.cells_given = args.cells is not None
    args.warmup = max(3, args.warmup)
    ws, rank, local = dist_env()
    if args.workload not in WORKLOADS:
        # accuracy/throughput reports for the other configurations (not the headline line)
        run = {"mms32": run_mms32, "plate20k": run_plate20k, "batch512": run_batch512, "serve": run_serve,
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
    out = run_workload(args.workload, args, ws, rank, local, not args.no_cpu, args.cells)
    if args.workload == "plate" and not args.no_wedge:
        w = run_workload("wedge", args, ws, rank, local, False, args.wedge_cells)
        out["wedge"] = {k: w[k] for k in ("value", "unit", "ms_per_step", "steps", "config", "roofline", "e2e",
                                          "clocks", "split_path", "df_path")}
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
