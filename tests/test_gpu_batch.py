"""Batched arena: several independent solves in one device arena, advanced by one
launch per kernel per stage for all of them.  Each instance must give bitwise the
results of its own single solve (same kernels, same per-cell arithmetic, same block
partition of its reductions), stop at its own limit, and keep a NaN to itself."""
import json

import numpy as np
import pytest

import ebbcfd_gb300 as E
from ebbcfd_gb300 import meshgen

pytestmark = pytest.mark.gpu

SIZES = [(800, 0.02, 0.3, 0.5), (3000, 0.08, 0.5, 0.6), (1500, 0.05, 0.7, 0.4), (6000, 0.1, 0.8, 0.5)]


def bump_cfg(mach, cfl, integrator="RK2_TVD", **kw):
    q = [mach, 0, 1, 1]
    d = {"mesh": "m.msh", "dt": 1e-4, "tEnd": 1000.0, "flux": "roeFlux", "saveIter": -1, "plotIter": -1,
         "forceBoundary": "Wall", "initialConditions": q, "integrator": integrator, "CFL": cfl,
         "boudaryConditions": [{"tag": "Inflow", "type": "fullState", "q": q},
                               {"tag": "Outflow", "type": "fullState", "q": q},
                               {"tag": "Wall", "type": "inviscidWall", "q": q}]}
    d.update(kw)
    return E.load_config(json.dumps(d))


@pytest.fixture(scope="module")
def instances():
    meshes = [meshgen.bump_channel(n, h=h, seed=k).to_solver_mesh() for k, (n, h, _, _) in enumerate(SIZES)]
    cfgs = [bump_cfg(m, c) for (_, _, m, c) in SIZES]
    return meshes, cfgs


def single_run(mesh, cfg, steps, precision):
    s = E.UfvmSolver(mesh, cfg, precision)
    rec = s.run(steps)
    out = s.state, s.time(), rec
    s.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_batch_equals_single_solves(instances, precision):
    meshes, cfgs = instances
    b = E.UfvmBatch(meshes, cfgs, precision)
    assert b.run(30, records=False) == 30
    st = b.status()
    whole = b.state
    for k, (m, c) in enumerate(zip(meshes, cfgs)):
        q, (t, dt, it), rec = single_run(m, c, 30, precision)
        qb = b.instance_state(k)
        assert np.array_equal(qb, q), (k, np.abs(qb - q).max())
        o = st[k]["cell_offset"]
        assert np.array_equal(whole[o:o + m.n_cells], q)
        assert st[k]["n_cells"] == m.n_cells
        assert (st[k]["t"], st[k]["dt"], st[k]["iterations"]) == (t, dt, it)
        assert st[k]["drag"] == rec[-1, 1] and st[k]["lift"] == rec[-1, 2]
        assert st[k]["resid"] == list(rec[-1, 3:7]) and st[k]["rmax"] == rec[-1, 7]
        assert st[k]["status"] == 0 and not st[k]["done"]
    b.close()


def test_each_instance_stops_at_its_own_limit(instances):
    meshes, cfgs = instances
    limits = [7, 25, 13, 40]
    b = E.UfvmBatch(meshes, cfgs)
    for k, n in enumerate(limits):
        b.set_stop(k, max_steps=n)
    assert b.run(1000, records=False) == max(limits)
    st = b.status()
    for k, n in enumerate(limits):
        assert st[k]["done"] and st[k]["iterations"] == n
        q, _, _ = single_run(meshes[k], cfgs[k], n, "fp64")
        assert np.array_equal(b.instance_state(k), q)
    b.close()


def test_residual_drop_retires_an_instance(instances):
    meshes, cfgs = instances
    _, _, rec = single_run(meshes[1], cfgs[1], 120, "fp64")
    rho = rec[:, 3]  # density residual
    drop = float(np.sort(rho / rho[0])[len(rho) // 3])
    expect = int(np.argmax(rho <= drop * rho[0])) + 1
    b = E.UfvmBatch(meshes[:2], cfgs[:2])
    b.set_stop(-1, max_steps=120)
    b.set_stop(1, max_steps=120, resid_drop=drop)
    b.run(1000, records=False)
    st = b.status()
    assert st[1]["done"] and st[1]["iterations"] == expect
    assert st[1]["resid_first"] == rho[0]
    assert st[0]["iterations"] == 120
    b.close()


def test_nan_halts_only_its_instance(instances):
    meshes, cfgs = instances
    b = E.UfvmBatch(meshes, cfgs)
    q1 = b.instance_state(1)
    q1[17, 0] = np.nan
    b.set_instance_state(1, q1)
    b.set_stop(-1, max_steps=12)
    b.run(100, records=False)
    st = b.status()
    assert st[1]["done"] and st[1]["status"] in (8, 9) and st[1]["err_index"] >= 0
    for k in (0, 2, 3):
        assert st[k]["status"] == 0 and st[k]["iterations"] == 12
        q, _, _ = single_run(meshes[k], cfgs[k], 12, "fp64")
        assert np.array_equal(b.instance_state(k), q)
    b.close()


def test_launch_and_sync_match_run(instances):
    meshes, cfgs = instances
    a = E.UfvmBatch(meshes, cfgs, "split")
    a.launch(20)
    a.sync()
    c = E.UfvmBatch(meshes, cfgs, "split")
    c.run(20, records=False)
    assert np.array_equal(a.state, c.state)
    assert [s["iterations"] for s in a.status()] == [20] * len(meshes)
    a.close()
    c.close()


def test_mixed_physics_is_rejected(instances):
    meshes, cfgs = instances
    other = bump_cfg(0.5, 0.5, integrator="RK4")
    with pytest.raises(E.EbbError) as ei:
        E.UfvmBatch(meshes[:2], [cfgs[0], other])
    assert ei.value.code == 5 and "share" in str(ei.value)


def test_footprint_matches_allocation(instances):
    meshes, cfgs = instances
    fp = E.batch_footprint(meshes, cfgs, "split")
    one = sum(E.batch_footprint([m], [c], "split") for m, c in zip(meshes, cfgs))
    assert 0.8 * one < fp < 1.2 * one


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_triangles_batched_with_polygons(instances, precision):
    """A triangle mesh batched with a mesh of quads, pentagons and a hexagon runs
    through the six-neighbour kernels (the padded slot rows of its cells are never
    used) and still gives bitwise its own three-neighbour solve."""
    meshes, cfgs = instances
    poly = meshgen.hanging_quads(12).to_solver_mesh()
    q = [0.5, 0, 1, 1]
    pcfg = E.load_config(json.dumps({
        "mesh": "m.msh", "dt": 1e-4, "tEnd": 1000.0, "flux": "roeFlux", "saveIter": -1, "plotIter": -1,
        "forceBoundary": "Freestream", "initialConditions": q, "integrator": "RK2_TVD", "CFL": 0.5,
        "boudaryConditions": [{"tag": "Freestream", "type": "fullState", "q": q}]}))
    qp = E.UfvmSolver(poly, pcfg, precision)
    rng = np.random.default_rng(3)
    start = qp.state * (1 + 0.02 * rng.uniform(-1, 1, qp.state.shape))  # a flow that moves
    qp.close()
    b = E.UfvmBatch([meshes[0], poly], [cfgs[0], pcfg], precision)
    b.set_instance_state(1, start)
    b.run(25, records=False)
    q0, _, _ = single_run(meshes[0], cfgs[0], 25, precision)
    assert np.array_equal(b.instance_state(0), q0)
    s = E.UfvmSolver(poly, pcfg, precision)
    s.set_state(start)
    s.run(25, records=False)
    assert np.array_equal(b.instance_state(1), s.state)
    assert np.abs(s.state - start).max() > 0
    s.close()
    b.close()
