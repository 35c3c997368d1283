"""Offline autotuner for the launch bounds of the FP32 (split) kernels.

The split kernels are bound by memory latency: how many warps an SM keeps in flight
decides their speed, and that is set at compile time by the minimum-blocks-per-SM
argument of __launch_bounds__ (it caps registers per thread; too low a cap spills).
For every candidate setting this builds a variant of the library (under
ebbcfd_gb300/_build/tune_<k>/, with -DEBB_*_MINB_F overrides), times each kernel
with ebb_profile_kernels (CUDA events on the solver stream, best of three rounds of
50 launches) on the seeded Mach 2.5 wedge in split precision, and keeps per kernel
the fastest setting.  The kernels are independent launches, so one build per row of
candidates measures all three at once.

  python -m ebbcfd_gb300.autotune [--cells N] [--out PATH]

writes the choice as a header (default ebbcfd_gb300/csrc/tuned.h) that kernels.cuh
includes; needs a GPU.
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CANDIDATES = {"cell": [8, 10, 12, 14], "flux": [10, 12, 16, 20], "update": [4, 6, 8, 8]}
MACRO = {"cell": "EBB_CELL_MINB_F", "flux": "EBB_FLUX_MINB_F", "update": "EBB_UPD_MINB_F"}


def _measure(row, cells):
    """Build variant `row` and print one JSON line of kernel times (child process)."""
    sys.path.insert(0, ROOT)
    from ebbcfd_gb300 import build as B
    B.OUT = os.path.join(HERE, "_build", "tune_%d" % row)
    B.LIB = os.path.join(B.OUT, "libebbgb300.so")
    B.CLI = os.path.join(B.OUT, "ebb-solve")
    setting = {k: v[row] for k, v in CANDIDATES.items()}
    B.CU["k_split.cu"] = B.CU["k_split.cu"] + ["-D%s=%d" % (MACRO[k], v) for k, v in setting.items()]
    B.build(force=True)
    import ctypes as C
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib, meshgen
    L = _lib.load()
    mesh = meshgen.wedge(cells, seed=0).to_solver_mesh()
    q = [2.5, 0, 1, 1]
    cfg = E.default_config()
    E.set_boundaries(cfg, [("Inflow", "fullState", q), ("Top", "fullState", q), ("Symmetry", "symmetry", q),
                           ("Ramp", "inviscidWall", q), ("Outflow", "fullState", q)])
    cfg.flux, cfg.integrator, cfg.cfl, cfg.ic[0], cfg.t_end = 0, 1, 0.4, 2.5, 1e9
    s = E.UfvmSolver(mesh, cfg, "split")
    s.run(5, records=False)
    ms = (C.c_double * 4)()
    best = None
    for _ in range(3):
        if L.ebb_profile_kernels(s.h, 50, ms):
            raise RuntimeError("profiling failed")
        best = list(ms) if best is None else [min(a, b) for a, b in zip(best, ms)]
    s.close()
    print(json.dumps({"row": row, "setting": setting,
                      "us": {"cell": 1e3 * best[0], "flux": 1e3 * best[1], "update": 1e3 * best[2]}}), flush=True)


def tune(cells=1_000_000, out=None):
    rows = []
    for row in range(len(CANDIDATES["cell"])):
        p = subprocess.run([sys.executable, "-m", "ebbcfd_gb300.autotune", "--row", str(row), "--cells", str(cells)],
                           cwd=ROOT, capture_output=True, text=True)
        if p.returncode:
            raise RuntimeError("variant %d failed:\n%s" % (row, p.stdout + p.stderr))
        rows.append(json.loads([ln for ln in p.stdout.splitlines() if ln.startswith("{")][-1]))
    choice, lines = {}, []
    for k in ("cell", "flux", "update"):
        times = {}
        for r in rows:
            v = r["setting"][k]
            times[v] = min(times.get(v, 1e30), r["us"][k])
        choice[k] = min(times, key=times.get)
        lines.append("// k_%s: " % k + ", ".join("%d blocks %.1f us" % (v, t) for v, t in sorted(times.items())))
    text = ["// Generated by ebbcfd_gb300/autotune.py: per-kernel device time of the FP32",
            "// kernels on the %d-cell seeded wedge (split precision) for each minimum number" % cells,
            "// of resident blocks per SM requested through __launch_bounds__."] + lines
    text += ["#pragma once"]
    for k in ("cell", "flux", "update"):
        text += ["#ifndef %s" % MACRO[k], "#define %s %d" % (MACRO[k], choice[k]), "#endif"]
    path = out or os.path.join(HERE, "csrc", "tuned.h")
    with open(path, "w") as f:
        f.write("\n".join(text) + "\n")
    return choice, rows


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=1_000_000)
    ap.add_argument("--row", type=int, default=-1)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    if a.row >= 0:
        _measure(a.row, a.cells)
    else:
        c, rows = tune(a.cells, a.out)
        print(json.dumps({"choice": c, "rows": rows}))
