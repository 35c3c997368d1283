"""Restatement of the reference's gmsh 2.2 ASCII reader and JSON config loader.

TEST INFRASTRUCTURE ONLY (part of the parity oracle, imported by tests/ and by
bench.py's CPU-baseline leg; never by the product package).

* ``parse_gmsh`` follows ``source/io.d:689-990`` (parseGmshMesh): section parsing,
  boundary-group bookkeeping including the split-group merge (io.d:910-942) with the
  reference's own ``ebb.math.sum`` (source/math.d:18-33, which drops elements for
  lists longer than 6), reordering of boundary nodes by physical tag (io.d:946-960)
  and the clockwise-element fix (io.d:969-987).
* ``load_config`` follows ``source/config.d:112-313`` (loadConfig): required keys,
  defaults, and "key present => value is JSON true" semantics for the flags.
"""
import json
import math

import numpy as np

BC_TYPES = {
    "fullState": 0,
    "constP": 1,
    "inviscidWall": 2,
    "viscidWall": 3,
    "symmetry": 4,
    "tpInflow": 5,
    "dirichlet": 6,
}
FLUXES = {"rusanovFlux": 0, "roeFlux": 1}
INTEGRATORS = {"Euler": 0, "RK2": 1, "RK2_TVD": 2, "RK4": 3}


def ebb_sum_lengths(groups):
    """source/math.d:18-33 applied as ``groups.sum!".length"``."""
    data = [len(g) for g in groups]

    def rec(d):
        if len(d) <= 6:
            s = d[0]
            for x in d[1:]:
                s += x
            return s
        m = int(math.floor(len(d) / 2.0))
        return rec(d[0:m - 1]) + rec(d[m:len(d) - 1])

    return rec(data)


def _clean(line):
    # io.d:662-666: strip, detab, split on ' ', drop empty tokens
    return [t for t in line.strip().replace("\t", " ").split(" ") if t != ""]


def parse_gmsh(path):
    """Return dict(nodes (N,2), elements list of 1-based node lists (CCW),
    bNodes (B,2) 0-based, bGroupStart list, bTags list)."""
    with open(path, "r") as f:
        lines = f.read().split("\n")
    pos = [0]

    def eof():
        return pos[0] >= len(lines)

    def readline():
        line = lines[pos[0]] if pos[0] < len(lines) else ""
        pos[0] += 1
        return _clean(line)

    nodes, elements, bTags = [], [], []
    bNodes, bGroups = [], []

    def end_section():
        t = readline()
        if not t or "$End" not in t[0]:
            raise ValueError("Expected section end")

    while not eof():
        t = readline()
        while len(t) == 0 and not eof():
            t = readline()
        if eof() and len(t) == 0:
            break
        if len(t) != 1 or t[0][0] != "$":
            raise ValueError("Incorrectly formatted section header")
        sec = t[0][1:]
        if sec == "MeshFormat":
            fmt = readline()
            if int(fmt[1]) != 0:
                raise ValueError("Unsupported mesh format")
            end_section()
        elif sec == "PhysicalNames":
            n = int(readline()[0])
            for _ in range(n):
                nl = readline()
                if len(nl) != 3:
                    raise ValueError("Expected 3 entries")
                if int(nl[0]) == 1:
                    bTags.append(nl[2].strip('"'))
            end_section()
        elif sec == "Nodes":
            n = int(readline()[0])
            for i in range(n):
                nl = readline()
                if int(nl[0]) != i + 1:
                    raise ValueError("Unexpected node number")
                nodes.append([float(x) for x in nl[1:-1]])
            end_section()
        elif sec == "Elements":
            n = int(readline()[0])
            cur = -1
            for i in range(n):
                el = [int(x) for x in readline()]
                if len(el) <= 4:
                    raise ValueError("Element line must have at least 4 entries")
                if el[0] != i + 1:
                    raise ValueError("Unexpected element number")
                etype, ntags = el[1], el[2]
                if ntags < 1:
                    raise ValueError("Expected at least one element tag")
                if etype == 1:
                    g = el[3]
                    bn = [x - 1 for x in el[3 + ntags:]]
                    if g != cur:
                        cur = g
                        bGroups.append([])
                    bGroups[-1].append(g)
                    bNodes.append(bn)
                elif etype in (2, 3):
                    elements.append(el[3 + ntags:])
                else:
                    raise ValueError("Unsupported element type: %d" % etype)
            end_section()
        else:
            while True:
                if eof():
                    raise ValueError("Unexpected end of file")
                tt = readline()
                if tt and "$End" in tt[0]:
                    break

    if len(bGroups) != len(bTags):
        newN, newG = [], []
        for i, g in enumerate(bGroups):
            cur = g[0]
            old = next((k for k, gg in enumerate(newG) if gg[0] == cur), -1)
            ns = 0 if i == 0 else ebb_sum_lengths(bGroups[0:i])
            ne = ebb_sum_lengths(bGroups[0:i + 1])
            if old >= 0:
                nne = ebb_sum_lengths(newG[0:old + 1])
                newG[old] = newG[old] + g
                newN = newN[0:nne] + bNodes[ns:ne] + newN[nne:]
            else:
                newG.append(list(g))
                newN = newN + bNodes[ns:ne]
        bNodes, bGroups = newN, newG
    if len(bGroups) != len(bTags):
        raise ValueError("Number of boundary groups does not match the number of boundary tags")

    outB, start = [], []
    for i in range(len(bGroups)):
        gi = next((k for k, gg in enumerate(bGroups) if gg[0] == i + 1), -1)
        if gi < 0:
            raise ValueError("Could not determine boundary group")
        ne = ebb_sum_lengths(bGroups[0:gi + 1])
        ns = 0 if gi == 0 else ebb_sum_lengths(bGroups[0:gi])
        start.append(len(outB))
        outB.extend(bNodes[ns:ne])

    xy = np.array(nodes, dtype=np.float64)
    for i, el in enumerate(elements):
        area = 0.0
        k = len(el)
        for j in range(k):
            n1, n2 = el[j] - 1, el[(j + 1) % k] - 1
            area += xy[n1, 0] * xy[n2, 1] - xy[n2, 0] * xy[n1, 1]
        if area < 0:
            elements[i] = el[::-1]
    return {
        "nodes": xy,
        "elements": elements,
        "bNodes": np.array(outB, dtype=np.int64).reshape(-1, 2),
        "bGroupStart": start,
        "bTags": bTags,
    }


def _get_double(v):
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise ValueError("invalid type")
    return float(v)


def load_config(text):
    """source/config.d:112-313.  Returns a plain dict."""
    j = json.loads(text)
    c = {}
    c["mesh"] = j["mesh"]
    c["flux"] = j["flux"]
    if not isinstance(j["dt"], float):
        raise ValueError("dt must be a floating-point JSON number")
    c["dt"] = j["dt"]
    c["tEnd"] = _get_double(j["tEnd"])
    c["saveIter"] = int(j["saveIter"])
    c["plotIter"] = int(j["plotIter"])
    fb = j.get("forceBoundary")
    c["forceBoundary"] = list(fb) if isinstance(fb, list) else [fb]

    def flag(key, default):
        return (j[key] is True) if key in j else default

    c["CFL"] = _get_double(j["CFL"]) if "CFL" in j else 0.5
    c["dynamicDt"] = flag("dynamicDt", True)
    c["integrator"] = j["integrator"] if "integrator" in j else "Euler"
    c["limited"] = flag("limited", True)
    c["localTimestep"] = flag("localTimestep", False)
    c["lpThresh"] = _get_double(j["lpThresh"]) if "lpThresh" in j else -1.0
    order = int(j["order"]) if "order" in j else 2
    c["order"] = order if order in (1, 2) else 2
    c["multistageLimiting"] = flag("multistageLimiting", True)
    c["cflAdjust"] = flag("cflAdjust", True)
    c["viscosity"] = flag("viscosity", False)
    pc = {"Pr": 0.7, "R": 8.3145, "gamma": 1.4, "Re": 1000.0, "L": 1.0}
    try:
        p = j["physicalConfig"]
        pc = {k: _get_double(p[k]) for k in ("Pr", "R", "gamma", "Re", "L")}
    except (KeyError, ValueError, TypeError):
        pass
    c["physicalConfig"] = pc
    ic = j["initialConditions"]
    c["ic"] = [_get_double(ic[k]) for k in range(4)]
    bcs = []
    for b in j["boudaryConditions"]:
        bcs.append({"tag": b["tag"], "type": BC_TYPES.get(b["type"], 0),
                    "q": [_get_double(x) for x in b["q"]]})
    c["boundaries"] = bcs
    return c
