"""Offline autotuner for the launch bounds of the solver kernels.

The split kernels are bound by memory latency: how many warps an SM keeps in flight
decides their speed, and that is set at compile time by the minimum-blocks-per-SM
argument of __launch_bounds__ (it caps registers per thread; too low a cap spills).
The FP64 kernels are bound by the FP64 pipe; a few more warps can still fill its
gaps, so they are tuned the same way.
For every row of candidate settings this builds a variant of the library (under
ebbcfd_gb300/_build/tune_<k>/, with -DEBB_*_MINB_* overrides), times each kernel of
both precision forms with ebb_profile_kernels (CUDA events on the solver stream, best
of three rounds) on the seeded Mach 2.5 wedge, and keeps per kernel the fastest
setting.  The kernels are independent launches, so one build per row measures all
six at once.  Register allocation does not change results: the FP64 kernels stay
bitwise equal to the oracle whatever the setting.

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
# per precision form and kernel: candidate minimum blocks per SM, one row per build
CANDIDATES = {"split": {"cell": [6, 8, 10, 12], "flux": [10, 12, 16, 20], "update": [4, 6, 8, 8]},
              "fp64": {"cell": [1, 5, 6, 8], "flux": [1, 5, 6, 8], "update": [1, 2, 3, 4]}}
MACRO = {("split", "cell"): "EBB_CELL_MINB_F", ("split", "flux"): "EBB_FLUX_MINB_F",
         ("split", "update"): "EBB_UPD_MINB_F", ("fp64", "cell"): "EBB_CELL_MINB_D",
         ("fp64", "flux"): "EBB_FLUX_MINB_D", ("fp64", "update"): "EBB_UPD_MINB_D"}
UNIT = {"split": "k_split.cu", "fp64": "k_fp64.cu"}
N_ROWS = 4


def _measure(row, cells):
    """Build variant `row` and print one JSON line of kernel times (child process)."""
    sys.path.insert(0, ROOT)
    from ebbcfd_gb300 import build as B
    B.OUT = os.path.join(HERE, "_build", "tune_%d" % row)
    B.LIB = os.path.join(B.OUT, "libebbgb300.so")
    B.CLI = os.path.join(B.OUT, "ebb-solve")
    setting = {p: {k: v[row] for k, v in c.items()} for p, c in CANDIDATES.items()}
    for p, st in setting.items():
        B.CU[UNIT[p]] = B.CU[UNIT[p]] + ["-D%s=%d" % (MACRO[(p, k)], v) for k, v in st.items()]
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
    us = {}
    for p in CANDIDATES:
        s = E.UfvmSolver(mesh, cfg, p)
        s.run(5, records=False)
        ms = (C.c_double * 4)()
        best = None
        for _ in range(3):
            if L.ebb_profile_kernels(s.h, 50 if p == "split" else 5, ms):
                raise RuntimeError("profiling failed")
            best = list(ms) if best is None else [min(a, b) for a, b in zip(best, ms)]
        s.close()
        us[p] = {"cell": 1e3 * best[0], "flux": 1e3 * best[1], "update": 1e3 * best[2]}
    print(json.dumps({"row": row, "setting": setting, "us": us}), flush=True)


def tune(cells=1_000_000, out=None):
    rows = []
    for row in range(N_ROWS):
        p = subprocess.run([sys.executable, "-m", "ebbcfd_gb300.autotune", "--row", str(row), "--cells", str(cells)],
                           cwd=ROOT, capture_output=True, text=True)
        if p.returncode:
            raise RuntimeError("variant %d failed:\n%s" % (row, p.stdout + p.stderr))
        rows.append(json.loads([ln for ln in p.stdout.splitlines() if ln.startswith("{")][-1]))
    choice, lines = {}, []
    for prec in CANDIDATES:
        for k in ("cell", "flux", "update"):
            times = {}
            for r in rows:
                v = r["setting"][prec][k]
                times[v] = min(times.get(v, 1e30), r["us"][prec][k])
            choice[(prec, k)] = min(times, key=times.get)
            lines.append("// %s k_%s: " % (prec, k) +
                         ", ".join("%d blocks %.1f us" % (v, t) for v, t in sorted(times.items())))
    text = ["// Generated by ebbcfd_gb300/autotune.py: per-kernel device time on the %d-cell seeded" % cells,
            "// wedge, both precision forms, for each minimum number of resident blocks per SM",
            "// requested through __launch_bounds__ (1 = the compiler's register choice)."] + lines
    text += ["#pragma once"]
    for key, m in MACRO.items():
        text += ["#ifndef %s" % m, "#define %s %d" % (m, choice[key]), "#endif"]
    path = out or os.path.join(HERE, "csrc", "tuned.h")
    with open(path, "w") as f:
        f.write("\n".join(text) + "\n")
    return {"%s/%s" % k: v for k, v in choice.items()}, rows


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
