"""ebb-solve command-line driver (app/solver.d semantics) on the GPU: files written,
their formats (.esln v2 per io.d:68-161, boundaryForces.frc per app/solver.d:184-192)
and their contents against the oracle's runIntegrator restatement."""
import json
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from ebbcfd_gb300 import build as B
from oracle import gmsh_ref, ref

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
MESHES = os.path.join(HERE, "golden", "meshes")


def read_esln(path):
    """Independent big-endian reader of .esln v2 (the layout of io.d:92-146)."""
    b = open(path, "rb").read()
    magic, ver, n = struct.unpack(">III", b[:12])
    t, dt = struct.unpack(">dd", b[12:28])
    M, order = struct.unpack(">II", b[28:36])
    off = 36
    q, faces, ids = [], [], []
    for _ in range(n):
        gid, ne = struct.unpack(">IB", b[off:off + 5])
        off += 5
        q.append(struct.unpack(">4d", b[off:off + 32]))
        off += 32
        faces.extend(struct.unpack(">4d", b[off + 32 * j:off + 32 * j + 32]) for j in range(ne))
        off += 32 * ne
        ids.append(gid)
    assert len(b) == off + 4  # CRC
    return {"magic": magic, "version": ver, "t": t, "dt": dt, "M": M, "order": order, "q": np.array(q),
            "faces": np.array(faces), "ids": ids}


def read_frc(path):
    b = open(path, "rb").read()
    assert len(b) % 24 == 0
    return np.array(struct.unpack(">%dd" % (len(b) // 8), b)).reshape(-1, 3)


@pytest.fixture()
def plate_dir(tmp_path):
    shutil.copy(os.path.join(MESHES, "flatPlate_0.msh"), tmp_path / "flatPlate_0.msh")
    d = json.load(open(os.path.join(MESHES, "flatPlate_0.json")))
    d["plotIter"] = 3
    d["saveIter"] = 4
    d["dt"] = 1e-5
    d["tEnd"] = 0.25
    (tmp_path / "cfg.json").write_text(json.dumps(d))
    return tmp_path, d


def test_ebb_solve_run_and_restart(plate_dir):
    B.build()
    tmp, d = plate_dir
    p = subprocess.run([B.CLI, "-c", "cfg.json"], cwd=tmp, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "Running 2D finite volume solver" in p.stdout and "-flux: roeFlux" in p.stdout
    frc = read_frc(tmp / "boundaryForces.frc")
    n = len(frc)
    assert n >= 9
    # the oracle runs the same loop
    conf = gmsh_ref.load_config(json.dumps(d))
    om = ref.OracleMesh(gmsh_ref.parse_gmsh(str(tmp / "flatPlate_0.msh")), conf)
    rec = om.run(10 ** 6)
    assert len(rec) == n
    # t column bitwise; drag and lift from differently ordered sums
    assert np.array_equal(frc[:, 0], rec[:, 0])
    assert np.abs(frc[:, 1:] - rec[:, 1:3]).max() <= 1e-9 * max(1.0, np.abs(rec[:, 1:3]).max())
    fin = read_esln(tmp / "final_0.esln")
    assert (fin["magic"], fin["version"], fin["M"], fin["order"]) == (0xEA98E1F5, 2, 4, 2)
    assert fin["ids"] == list(range(len(fin["q"])))
    qo = om.state()
    scale = np.abs(qo).max(axis=0)
    assert (np.abs(fin["q"] - qo).max(axis=0) / scale).max() <= 1e-9  # constP ghosts use pow()
    assert fin["t"] == om.t and fin["dt"] == om.dt
    of = om.face_states()
    assert (np.abs(fin["faces"] - of).max(axis=0) / np.abs(of).max(axis=0)).max() <= 1e-9
    # save files every saveIter iterations, including iteration 0
    saves = sorted(f for f in os.listdir(tmp) if f.startswith("save_"))
    assert saves == ["save_%d_0.esln" % k for k in range((n - 1) // 4 + 1)]
    s1 = read_esln(tmp / "save_1_0.esln")
    assert s1["t"] == rec[4, 0] and s1["dt"] == rec[4, 8]
    # restart from save_1_ continues at that t
    p2 = subprocess.run([B.CLI, "-c", "cfg.json", "-s", "save_1_"], cwd=tmp, capture_output=True, text=True,
                        timeout=300)
    assert p2.returncode == 0, p2.stdout + p2.stderr
    frc2 = read_frc(tmp / "boundaryForces.frc")
    assert frc2[0, 0] == s1["t"]
    fin2 = read_esln(tmp / "final_0.esln")
    assert fin2["t"] >= d["tEnd"]


def test_ebb_solve_precision_forms(plate_dir):
    """`--precision df` runs the same loop in double-float: the same number of records,
    times and final state within 1e-9 of the oracle's (relative to each component's
    largest magnitude).  `--precision split` runs it too (its time steps, from FP32
    wave speeds, may end the loop one step apart); an unknown form is refused."""
    B.build()
    tmp, d = plate_dir
    conf = gmsh_ref.load_config(json.dumps(d))
    om = ref.OracleMesh(gmsh_ref.parse_gmsh(str(tmp / "flatPlate_0.msh")), conf)
    rec = om.run(10 ** 6)
    qo = om.state()
    for form in ("df", "split"):
        p = subprocess.run([B.CLI, "-c", "cfg.json", "--precision", form], cwd=tmp, capture_output=True, text=True,
                           timeout=300)
        assert p.returncode == 0, p.stdout + p.stderr
        frc = read_frc(tmp / "boundaryForces.frc")
        if form == "split":
            assert abs(len(frc) - len(rec)) <= 1
            continue
        assert len(frc) == len(rec)
        assert np.abs(frc[:, 0] - rec[:, 0]).max() <= 1e-9 * rec[-1, 0]
        fin = read_esln(tmp / "final_0.esln")
        assert (np.abs(fin["q"] - qo).max(axis=0) / np.abs(qo).max(axis=0)).max() <= 1e-9
    bad = subprocess.run([B.CLI, "-c", "cfg.json", "--precision", "fp16"], cwd=tmp, capture_output=True, text=True,
                         timeout=60)
    assert bad.returncode == 2 and "unknown precision form" in bad.stderr


def test_ebb_solve_reports_missing_tag(tmp_path):
    B.build()
    shutil.copy(os.path.join(MESHES, "flatPlate_0.msh"), tmp_path / "flatPlate_0.msh")
    d = json.load(open(os.path.join(MESHES, "flatPlate_0.json")))
    d["boudaryConditions"] = d["boudaryConditions"][:2]
    (tmp_path / "cfg.json").write_text(json.dumps(d))
    p = subprocess.run([B.CLI, "-c", "cfg.json"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert p.returncode == 1 and "Could not find matching boundary condition tag" in p.stdout


def test_esln_file_is_the_one_the_reference_reader_checked(tmp_path):
    """The library's .esln writer gives, byte for byte, the committed fixture that the
    reference's own reader (scripts/python/EbbUtils.py:7-77, run when the fixture was
    made by tests/golden/make_esln_fixture.py) parsed into the oracle's state, global
    ids, edge counts and face states."""
    import hashlib
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_esln_fixture as F
    chk = json.load(open(F.CHECK))
    out = tmp_path / "again.esln"
    F.write(str(out))
    data = out.read_bytes()
    assert hashlib.sha256(data).hexdigest() == chk["sha256"]
    assert data == open(F.FIXTURE, "rb").read()
    r = read_esln(str(out))
    assert r["version"] == 2 and r["M"] == 4 and len(r["q"]) == chk["found"]["n_cells"]
