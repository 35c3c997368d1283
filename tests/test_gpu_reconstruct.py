"""ebb-reconstruct (app/reconstruct.d:79-424) on the GPU against the oracle's
restatement: node, edge and cell values of the refined mesh, and the .mmsh / .esln
files the CLI writes."""
import json
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from ebbcfd_gb300 import build as B
from oracle import gmsh_ref, ref
from tests import cases

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
MESHES = os.path.join(HERE, "golden", "meshes")
USES_POW = {"flatplate_ns"}  # constant-pressure ghosts use pow()


@pytest.mark.parametrize("name", ["wedge_rusanov", "flatplate_ns", "sine_quads_tvd", "mms_tri_pert_lp",
                                  "plate_ns_rk4"])
def test_reconstruct_matches_oracle(name):
    c = cases.case(name)
    sol, om = c.build()
    sol.run(7, records=False)
    om.run(7)
    q = sol.reconstruct()
    nv, ev, cv = om.reconstruct()
    want = np.vstack([nv, ev, cv])
    assert q.shape == want.shape
    if name in USES_POW:
        scale = np.maximum(np.abs(want).max(axis=0), 1e-300)
        assert (np.abs(q - want).max(axis=0) / scale).max() <= 1e-12
    else:
        assert np.array_equal(q, want), np.abs(q - want).max()


def test_reconstruct_split_precision_close():
    c = cases.case("wedge_rusanov")
    sol, om = c.build()
    import ebbcfd_gb300 as E
    sol.run(20, records=False)
    s2 = E.UfvmSolver(sol.mesh, sol.cfg, "split")
    s2.set_state(sol.state)
    q64 = sol.reconstruct()
    q32 = s2.reconstruct()
    scale = np.abs(q64).max(axis=0)
    assert (np.abs(q32 - q64).max(axis=0) / scale).max() < 1e-5


def _read_mmsh(path):
    b = open(path, "rb").read()
    off = 0

    def u64():
        nonlocal off
        v = struct.unpack(">Q", b[off:off + 8])[0]
        off += 8
        return v
    n = u64()
    pts = np.array(struct.unpack(">%dd" % (2 * n), b[off:off + 16 * n])).reshape(n, 2)
    off += 16 * n
    m = u64()
    tris = np.array(struct.unpack(">%dd" % (3 * m), b[off:off + 24 * m])).reshape(m, 3)
    off += 24 * m
    assert (u64(), u64(), u64()) == (0, 0, 0) and off == len(b)
    return pts, tris


def test_ebb_reconstruct_cli(tmp_path):
    B.build()
    shutil.copy(os.path.join(MESHES, "flatPlate_0.msh"), tmp_path / "flatPlate_0.msh")
    d = json.load(open(os.path.join(MESHES, "flatPlate_0.json")))
    d.update({"plotIter": 5, "saveIter": 5, "dt": 1e-5, "tEnd": 0.2})
    (tmp_path / "cfg.json").write_text(json.dumps(d))
    p = subprocess.run([B.CLI, "-c", "cfg.json"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    p = subprocess.run([B.RECON, "cfg.json", "save_1_0.esln"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "saveNum: 1" in p.stdout
    pts, tris = _read_mmsh(tmp_path / "recon_flatPlate_0.mmsh")
    # the oracle from the same saved state
    conf = gmsh_ref.load_config(json.dumps(d))
    mesh = gmsh_ref.parse_gmsh(str(tmp_path / "flatPlate_0.msh"))
    om = ref.OracleMesh(mesh, conf)
    from tests import test_gpu_cli as cli
    sv = cli.read_esln(tmp_path / "save_1_0.esln")
    om.set_state(sv["q"])
    nv, ev, cv = om.reconstruct()
    rs = cli.read_esln(tmp_path / "recon_save_1.esln")
    assert (rs["t"], rs["dt"]) == (sv["t"], sv["dt"]) and rs["ids"] == list(range(len(rs["q"])))
    want = np.vstack([nv, ev, cv])
    scale = np.abs(want).max(axis=0)
    assert (np.abs(rs["q"] - want).max(axis=0) / scale).max() <= 1e-12
    assert len(pts) == len(want) and len(rs["faces"]) == 0
    n_slots = sum(len(e) for e in mesh["elements"])
    assert len(tris) == 2 * n_slots and tris.min() >= 1 and tris.max() <= len(pts)
    # points: used nodes, then edge midpoints, then the cell centroids
    import ebbcfd_gb300 as E
    cen = E.import_mesh(str(tmp_path / "flatPlate_0.msh")).centroids()
    assert np.array_equal(pts[len(nv) + len(ev):], cen)
    assert np.array_equal(pts[:len(nv)], mesh["nodes"][:len(nv), :2])  # every node of this mesh is used
