#!/usr/bin/env python3
"""The .esln fixture checked with the reference's own reader.

Two steps, on two machines:

1. On a machine with a GPU, the library writes the solution file of a small parity
   case after 10 steps (plain FP64, bitwise equal to the oracle):

       python tests/golden/make_esln_fixture.py --write <file.esln>

2. Where the EbbCFD tree is available (its Python scripts import here; it is never
   read at test time), the reference's reader scripts/python/EbbUtils.py
   (importEbbSolution, EbbUtils.py:7-77) parses that file, and its cell averages,
   global ids, edge counts and per-edge values are compared with the oracle's state
   and face states after the same 10 steps:

       python tests/golden/make_esln_fixture.py --check <file.esln> --ref <EbbCFD tree>

   On a match the file is copied to tests/golden/esln/ with reader_check.json (its
   sha256 and what the reference's reader found).  The GPU test then writes the same
   solution again and compares it byte for byte with the fixture.

The reference's force-file reader (importEbbForces, EbbUtils.py:141-159) is Python 2
code: under Python 3 it fails at np.zeros with a float size, so .frc files are checked
by the tests' own big-endian (t, drag, lift) parser instead.
"""
import argparse
import hashlib
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASE = "mms_tri_limited"
STEPS = 10
FIXTURE = os.path.join(HERE, "esln", "%s_%d.esln" % (CASE, STEPS))
CHECK = os.path.join(HERE, "esln", "reader_check.json")


def write(path):
    sys.path.insert(0, ROOT)
    from tests.cases import case
    sol, _ = case(CASE).build()
    sol.run(STEPS, records=False)
    sol.save_solution(path)
    sol.close()


def check(path, ref):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ref, "scripts", "python"))
    import EbbUtils  # the reference's reader
    from oracle import gmsh_ref, ref as oracle_ref
    from tests.cases import case
    sln = EbbUtils.importEbbSolution(path)
    c = case(CASE)
    om = oracle_ref.OracleMesh(c.reader_mesh(), gmsh_ref.load_config(c.text), mms=c.mms)
    om.run(STEPS)
    q = om.state()
    faces = om.face_states()
    nedge = [len(e) for e in case(CASE).reader_mesh()["elements"]]
    edge_vals = np.array([v for cell in sln["edgeVals"] for v in cell])
    found = {
        "version": sln["version"], "M": sln["M"], "order": sln["order"], "n_cells": len(sln["U"]),
        "cell_averages_equal_oracle_state": bool(np.array_equal(np.asarray(sln["U"]), q)),
        "global_ids_in_cell_order": bool(list(sln["gens"]) == list(range(len(q)))),
        "edge_counts_equal_elements": bool(list(sln["edges"]) == nedge),
        "edge_values_equal_oracle_face_states": bool(edge_vals.shape == faces.shape and np.array_equal(edge_vals, faces)),
    }
    if not all(v for k, v in found.items() if isinstance(v, bool)) or found["version"] != 2:
        raise SystemExit("the reference's reader disagrees with the oracle: %s" % found)
    os.makedirs(os.path.dirname(FIXTURE), exist_ok=True)
    shutil.copyfile(path, FIXTURE)
    out = {"reader": "scripts/python/EbbUtils.py:7-77 importEbbSolution", "case": CASE, "steps": STEPS,
           "file": os.path.basename(FIXTURE), "sha256": hashlib.sha256(open(FIXTURE, "rb").read()).hexdigest(),
           "found": found}
    json.dump(out, open(CHECK, "w"), indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--write")
    ap.add_argument("--check")
    ap.add_argument("--ref")
    a = ap.parse_args()
    if a.write:
        write(a.write)
    elif a.check and a.ref:
        check(a.check, a.ref)
    else:
        ap.error("--write FILE, or --check FILE --ref TREE")
