"""Offline autotuner for the launch shape of the solver kernels.

Two dimensions per kernel are searched: threads per block and the minimum resident
blocks per SM requested through __launch_bounds__.  The split kernels are bound by
memory latency, so the warps an SM keeps in flight decide their speed; the block
size and the minimum-blocks argument (a cap on registers per thread -- too low a cap
spills) set that at compile time.  The FP64 kernels are bound by the FP64 pipe; a few
more warps can still fill its gaps.  The double-float kernels run long dependent FP32
sequences with many live values: few warps, and a cap that does not spill.  k_update's block size (256 or 512) is also the
size of the per-block reduction trees and of the batched arena's update-block map, so
one value serves all precision forms in a build.

Every row of candidate settings is one variant of the library (under
ebbcfd_gb300/_build/tune_<k>/, with -DEBB_* overrides; the variants compile in
parallel).  Each variant's kernels of the three precision forms are timed with
ebb_profile_kernels (CUDA events on the solver stream, best of three rounds) on the
headline workload -- the 4.0M-cell Navier-Stokes plate (--workload wedge: the 1.0M
Mach 2.5 wedge) -- and per kernel the fastest setting over the rows is kept.  The
kernels are independent launches, so one variant measures all of them at once.  Split
precision has two launch-shape profiles: viscous meshes (gradients stored, the
viscous flux) take the shapes timed on the tuned workload, inviscid meshes their own,
timed on the wedge.  Register
allocation and block size change no FP64 result bit (the kernels stay bitwise equal to
the oracle); the update block size changes the order of the RMS residual sums only.

  python -m ebbcfd_gb300.autotune [--workload plate|wedge] [--cells N] [--out PATH]

writes the choice as a header (default ebbcfd_gb300/csrc/tuned.h) that kernels.cuh
includes, with every row's timings in its comments; needs a GPU.
"""
import argparse
import json
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# per precision form and kernel: candidate (threads per block, minimum blocks per SM),
# one entry per row (threads x blocks <= 2048); the update kernel's threads come from
# UPD_TB, shared by all forms
CANDIDATES = {
    "split": {"cell": [(128, 8), (128, 10), (128, 6), (256, 4), (256, 3), (64, 16), (64, 12)],
              "flux": [(128, 12), (128, 10), (128, 8), (256, 6), (256, 4), (64, 20), (64, 16)],
              "update": [8, 6, 4, 4, 3, 8, 2]},
    "fp64": {"cell": [(128, 5), (128, 1), (128, 6), (256, 2), (256, 3), (64, 8), (64, 10)],
             "flux": [(128, 1), (128, 4), (128, 5), (256, 2), (256, 1), (64, 8), (64, 6)],
             "update": [3, 1, 2, 2, 1, 4, 1]},
    "df": {"cell": [(128, 2), (128, 1), (128, 3), (256, 1), (256, 2), (64, 4), (64, 6)],
           "flux": [(128, 2), (128, 1), (128, 3), (256, 1), (256, 2), (64, 4), (64, 6)],
           "update": [3, 1, 2, 2, 1, 4, 1]},
    # split precision on inviscid meshes (its own launch-shape profile, timed on the wedge)
    "split_inv": {"cell": [(128, 8), (128, 10), (128, 6), (256, 4), (256, 3), (64, 16), (64, 12)],
                  "flux": [(128, 12), (128, 10), (128, 8), (256, 6), (256, 4), (64, 20), (64, 16)],
                  "update": [8, 6, 4, 4, 3, 8, 2]},
}
# the form each candidate set is built and timed in, and on which workload (None: the
# workload being tuned for)
FORM = {"split": ("split", None), "fp64": ("fp64", None), "df": ("df", None), "split_inv": ("split", "wedge")}
UPD_TB = [256, 256, 256, 512, 512, 256, 512]
N_ROWS = len(UPD_TB)
MACRO = {("split", "cell"): ("EBB_CELL_TB_F", "EBB_CELL_MINB_F"), ("split", "flux"): ("EBB_FLUX_TB_F", "EBB_FLUX_MINB_F"),
         ("fp64", "cell"): ("EBB_CELL_TB_D", "EBB_CELL_MINB_D"), ("fp64", "flux"): ("EBB_FLUX_TB_D", "EBB_FLUX_MINB_D"),
         ("df", "cell"): ("EBB_CELL_TB_W", "EBB_CELL_MINB_W"), ("df", "flux"): ("EBB_FLUX_TB_W", "EBB_FLUX_MINB_W"),
         ("split", "update"): ("EBB_UPD_TB", "EBB_UPD_MINB_F"), ("fp64", "update"): ("EBB_UPD_TB", "EBB_UPD_MINB_D"),
         ("df", "update"): ("EBB_UPD_TB", "EBB_UPD_MINB_W"),
         ("split_inv", "cell"): ("EBB_CELL_TB_FI", "EBB_CELL_MINB_FI"),
         ("split_inv", "flux"): ("EBB_FLUX_TB_FI", "EBB_FLUX_MINB_FI"),
         ("split_inv", "update"): ("EBB_UPD_TB", "EBB_UPD_MINB_FI")}


def setting(row):
    """{precision: {kernel: (threads, min blocks)}} of candidate row `row`."""
    out = {}
    for p, c in CANDIDATES.items():
        out[p] = {"cell": tuple(c["cell"][row]), "flux": tuple(c["flux"][row]), "update": (UPD_TB[row], c["update"][row])}
        for k, (tb, mb) in out[p].items():
            assert tb * mb <= 2048, (p, k, tb, mb)
    return out


def defines(row):
    d = {}
    for (p, k), (mt, mb) in MACRO.items():
        tb, b = setting(row)[p][k]
        d[mt] = tb
        d[mb] = b
    return ["-D%s=%d" % kv for kv in sorted(d.items())]


def _module(row):
    sys.path.insert(0, ROOT)
    from ebbcfd_gb300 import build as B
    B.OUT = os.path.join(HERE, "_build", "tune_%d" % row)
    B.LIB = os.path.join(B.OUT, "libebbgb300.so")
    B.CLI = os.path.join(B.OUT, "ebb-solve")
    B.RECON = os.path.join(B.OUT, "ebb-reconstruct")
    B.DEFINES = defines(row)
    return B


def _build(row):
    """Compile variant `row` (child process: the build module's paths are globals)."""
    _module(row).build(force=True)


def _measure(row, workload, cells):
    """Time variant `row`'s kernels; print one JSON line (child process)."""
    _module(row)
    import ctypes as C
    import ebbcfd_gb300 as E
    from ebbcfd_gb300 import _lib
    sys.path.insert(0, ROOT)
    import bench
    L = _lib.load(build_if_missing=False)
    meshes = {}
    us = {}
    for p in CANDIDATES:
        prec, wname = FORM[p]
        wname = wname or workload
        wl = bench.WORKLOADS[wname]
        if wname not in meshes:
            meshes[wname] = bench.make_mesh(wname, cells if wname == workload and cells else wl["cells"]).to_solver_mesh()
        s = E.UfvmSolver(meshes[wname], E.load_config(wl["config"]()), prec)
        s.run(5, records=False)
        ms = (C.c_double * 4)()
        best = None
        for _ in range(3):
            if L.ebb_profile_kernels(s.h, {"split": 20, "df": 6, "fp64": 3}[prec], ms):
                raise RuntimeError("profiling failed")
            best = list(ms) if best is None else [min(a, b) for a, b in zip(best, ms)]
        s.close()
        us[p] = {"cell": 1e3 * best[0], "flux": 1e3 * best[1], "update": 1e3 * best[2]}
    print(json.dumps({"row": row, "setting": setting(row), "us": us}), flush=True)


def tune(workload="plate", cells=None, out=None):
    def child(args):
        p = subprocess.run([sys.executable, "-m", "ebbcfd_gb300.autotune"] + args, cwd=ROOT, capture_output=True,
                           text=True)
        if p.returncode:
            raise RuntimeError("%s failed:\n%s" % (args, (p.stdout + p.stderr)[-3000:]))
        return p.stdout

    with ThreadPoolExecutor(max_workers=N_ROWS) as ex:
        list(ex.map(lambda r: child(["--build-row", str(r)]), range(N_ROWS)))
    rows = []
    for r in range(N_ROWS):
        o = child(["--row", str(r), "--workload", workload] + (["--cells", str(cells)] if cells else []))
        rows.append(json.loads([ln for ln in o.splitlines() if ln.startswith("{")][-1]))
    choice, lines = {}, []
    for prec in CANDIDATES:
        for k in ("cell", "flux", "update"):
            times = {}
            for r in rows:
                v = tuple(r["setting"][prec][k])
                times[v] = min(times.get(v, 1e30), r["us"][prec][k])
            choice[(prec, k)] = min(times, key=times.get)
            lines.append("// %s k_%s: " % (prec, k) +
                         ", ".join("%dx%d %.1f us" % (tb, b, t) for (tb, b), t in sorted(times.items())))
    # one update block size for all forms: the one whose best total is smaller
    upd = {}
    for tb in sorted(set(UPD_TB)):
        upd[tb] = sum(min(r["us"][p]["update"] for r in rows if r["setting"][p]["update"][0] == tb)
                      for p in CANDIDATES)
    tb_upd = min(upd, key=upd.get)
    for p in CANDIDATES:
        best = min((r["us"][p]["update"], tuple(r["setting"][p]["update"])) for r in rows
                   if r["setting"][p]["update"][0] == tb_upd)
        choice[(p, "update")] = best[1]
    cells_txt = "%d-cell" % cells if cells else "default-size"
    text = ["// Generated by ebbcfd_gb300/autotune.py on the %s %s workload: device time per" % (cells_txt, workload),
            "// launch of each kernel of the three precision forms for each (threads per block) x (minimum",
            "// resident blocks per SM requested through __launch_bounds__; 1 = the compiler's",
            "// register choice), best of three rounds of CUDA-event timing; fastest kept."] + lines
    text += ["// update block size %d (summed best update times: %s)" %
             (tb_upd, ", ".join("%d: %.1f us" % kv for kv in sorted(upd.items()))), "#pragma once"]
    for (p, k), (mt, mb) in MACRO.items():
        tb, b = choice[(p, k)]
        if k != "update" or p == "split":  # one update block size (EBB_UPD_TB) for all
            text += ["#ifndef %s" % mt, "#define %s %d" % (mt, tb), "#endif"]
        text += ["#ifndef %s" % mb, "#define %s %d" % (mb, b), "#endif"]
    path = out or os.path.join(HERE, "csrc", "tuned.h")
    with open(path, "w") as f:
        f.write("\n".join(text) + "\n")
    return {"%s/%s" % k: v for k, v in choice.items()}, rows


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="plate", choices=["plate", "wedge"])
    ap.add_argument("--cells", type=int, default=None)
    ap.add_argument("--row", type=int, default=-1)
    ap.add_argument("--build-row", type=int, default=-1)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    if a.build_row >= 0:
        _build(a.build_row)
    elif a.row >= 0:
        _measure(a.row, a.workload, a.cells)
    else:
        c, rows = tune(a.workload, a.cells, a.out)
        print(json.dumps({"choice": c, "rows": rows}))
