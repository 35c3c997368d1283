#!/usr/bin/env python3
"""Regenerate the committed golden fixtures under tests/golden/ from the EbbCFD tree.

Run where the EbbCFD tree is available, giving its location:

    python tests/golden/make_golden.py --ref <EbbCFD tree>

Outputs (all committed; nothing at test time reads the reference tree):
  roe_kat.json        the four Roe-flux known answers of source/flux.d:143-219,
                      parsed from the unittest block as text (points, normal, F).
  published_l2.json   the MMS L2(rho) and flat-plate Cd values tabulated in
                      ms_refinement/plot_conv.py:6-20.
  meshes/*.msh, *.json  the reference's own MMS and flat-plate fixture meshes and
                      configs, copied byte for byte, with sha256 in manifest.json.
"""
import argparse
import hashlib
import json
import os
import re
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))

MESHES = [
    "ms_refinement/ms_refine_0.msh", "ms_refinement/ms_refine_1.msh", "ms_refinement/ms_refine_2.msh",
    "ms_refinement/ms_refine_3.msh", "ms_refinement/ms_refine_tri_0.msh", "ms_refinement/ms_refine_tri_1.msh",
    "ms_refinement/ms_refine_tri_2.msh", "ms_refinement/ms_refine_tri_3.msh",
    "ms_refinement/ms_refine_tri_pert_0.msh", "ms_refinement/ms_refine_tri_pert_1.msh",
    "ms_refinement/ms_refine_tri_pert_2.msh", "flatPlate/flatPlate_0.msh", "flatPlate/flatPlate_1.msh",
]
CONFIGS = [
    "ms_refinement/ms_refine_0.json", "ms_refinement/ms_refine_3.json", "ms_refinement/ms_refine_vs_0.json",
    "ms_refinement/ms_refine_tri_0.json", "flatPlate/flatPlate_0.json", "flatPlate/flatPlate_1.json",
]


def parse_roe_kat(flux_d):
    text = open(flux_d).read()
    start = text.index("unittest")
    block = text[start:text.index("roeFlux(size_t dims)", start)]
    cases = []
    # each case: x1 = ..; y1 = ..; x2 = ..; y2 = ..; n = Vector!2(..); 4 writeln(abs(F[k] - v))
    parts = re.split(r"F = roeFlux!4\(qL, qR, n, sMax\);", block)
    pre = parts[0]
    for i in range(1, len(parts)):
        head = parts[i - 1]
        body = parts[i]
        def last(name, s):
            v = re.findall(name + r"\s*=\s*([-0-9.]+);", s)
            return float(v[-1])
        x1, y1, x2, y2 = last("x1", head), last("y1", head), last("x2", head), last("y2", head)
        nm = re.findall(r"n = Vector!2\(([^)]*)\)", head)[-1]
        if "sqrt" in nm:
            n = [2.0 ** 0.5 / 2.0, 2.0 ** 0.5 / 2.0]
        else:
            n = [float(t) for t in nm.split(",")]
        F = [float(v) for v in re.findall(r"abs\(F\[\d\] - ([-0-9.]+)\)", body)[:4]]
        cases.append({"p1": [x1, y1], "p2": [x2, y2], "n": n, "F": F})
        pre = body
    return cases


def parse_plot_conv(path):
    out = {}
    for line in open(path):
        m = re.match(r"^(rl2_\w+|dx\w*|fp_actual)\s*=\s*(.*)$", line.strip())
        if m and "abs(" not in m.group(2):
            out[m.group(1)] = eval(m.group(2), {"sqrt": lambda v: v ** 0.5})
    m = re.search(r"rl2_ns_fp = \[(.*)\]", open(path).read())
    out["cd_flat_plate"] = [float(v) for v in re.findall(r"fp_actual - ([0-9.]+)", m.group(1))]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the EbbCFD source tree")
    a = ap.parse_args()
    kat = parse_roe_kat(os.path.join(a.ref, "source", "flux.d"))
    assert len(kat) == 4 and all(len(c["F"]) == 4 for c in kat), kat
    json.dump({"source": "source/flux.d:143-219", "fields": "source/manufacturedsolution.d:27-45",
               "cases": kat}, open(os.path.join(HERE, "roe_kat.json"), "w"), indent=1)
    pub = parse_plot_conv(os.path.join(a.ref, "ms_refinement", "plot_conv.py"))
    pub["source"] = "ms_refinement/plot_conv.py:6-20"
    json.dump(pub, open(os.path.join(HERE, "published_l2.json"), "w"), indent=1)
    os.makedirs(os.path.join(HERE, "meshes"), exist_ok=True)
    man = {}
    for rel in MESHES + CONFIGS:
        src = os.path.join(a.ref, rel)
        dst = os.path.join(HERE, "meshes", os.path.basename(rel))
        shutil.copyfile(src, dst)
        man[os.path.basename(rel)] = {"from": rel, "sha256": hashlib.sha256(open(dst, "rb").read()).hexdigest()}
    json.dump(man, open(os.path.join(HERE, "meshes", "manifest.json"), "w"), indent=1)
    print("wrote", len(kat), "KAT cases,", len(man), "fixture files")


if __name__ == "__main__":
    main()
