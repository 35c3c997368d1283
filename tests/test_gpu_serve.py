"""Request server: solves submitted while others run are admitted into arenas as
memory frees up, overlap on the device, and each result is bitwise the result of
solving that request alone with the same stop conditions."""
import json

import numpy as np
import pytest

import ebbcfd_gb300 as E
from ebbcfd_gb300 import meshgen

pytestmark = pytest.mark.gpu


def bump_cfg(mach, flux="roeFlux", rho=1.0):
    q = [mach, 0, 1, rho]
    return E.load_config(json.dumps({
        "mesh": "m.msh", "dt": 1e-4, "tEnd": 1000.0, "flux": flux, "saveIter": -1, "plotIter": -1,
        "forceBoundary": "Wall", "initialConditions": q, "integrator": "RK2_TVD", "CFL": 0.5,
        "boudaryConditions": [{"tag": "Inflow", "type": "fullState", "q": q},
                              {"tag": "Outflow", "type": "fullState", "q": q},
                              {"tag": "Wall", "type": "inviscidWall", "q": q}]}))


def cylinder_cfg(re, mach=0.2):
    q = [mach, 0, 1, 1]
    far = [{"tag": t, "type": "fullState", "q": q} for t in ("Inflow", "Outflow", "Top", "Bottom")]
    return E.load_config(json.dumps({
        "mesh": "m.msh", "dt": 1e-4, "tEnd": 1000.0, "flux": "roeFlux", "saveIter": -1, "plotIter": -1,
        "forceBoundary": "Cylinder", "initialConditions": q, "integrator": "RK2_TVD", "CFL": 0.5,
        "viscosity": True, "physicalConfig": {"Pr": 0.72, "R": 1.0, "gamma": 1.4, "Re": re, "L": 1.0},
        "boudaryConditions": far + [{"tag": "Cylinder", "type": "viscidWall", "q": q}]}))


@pytest.fixture(scope="module")
def requests():
    out = []
    for k, (kind, n, p, steps) in enumerate([("bump", 800, 0.3, 40), ("bump", 3000, 0.5, 64),
                                              ("cyl", 1000, 80.0, 33), ("bump", 1500, 0.7, 50),
                                              ("cyl", 3000, 150.0, 48), ("bump", 6000, 0.8, 70),
                                              ("bump", 2500, 0.6, 0)]):
        if kind == "bump":
            m, c = meshgen.bump_channel(n, h=0.05, seed=k).to_solver_mesh(), bump_cfg(p)
        else:
            m, c = meshgen.cylinder(n, seed=k).to_solver_mesh(), cylinder_cfg(p)
        out.append((m, c, steps))
    return out


def solo(mesh, cfg, max_steps, resid_drop, precision):
    s = E.UfvmSolver(mesh, cfg, precision)
    s.set_stop(0, t_end=cfg.t_end, max_steps=max_steps, resid_drop=resid_drop)
    s.run(10 ** 6, records=False)
    out = s.state, s.status()[0]
    s.close()
    return out


def serve(requests, precision, **opts):
    sv = E.EbbServer(precision, **opts)
    ids = {}
    drop = 0.5  # the request without a step limit stops at a residual drop
    for k, (m, c, steps) in enumerate(requests[:3]):
        ids[sv.submit(m, c, steps, 0.0 if steps else drop)] = k
    results = {}
    for _ in range(3):
        sv.tick()
    for k, (m, c, steps) in enumerate(requests[3:], start=3):
        ids[sv.submit(m, c, steps, 0.0 if steps else drop)] = k
    for _ in range(100000):
        a, w = sv.tick()
        for r in sv.results():
            results[ids[r["id"]]] = (r, sv.take_state(r["id"]))
        if len(results) == len(requests) and a == 0 and w == 0:
            break
    stats = sv.stats()
    sv.close()
    return results, stats, drop


@pytest.mark.parametrize("precision", ["split", "fp64"])
def test_served_results_equal_solo_solves(requests, precision):
    results, stats, drop = serve(requests, precision, max_batch=3, tick_ms=1.0, build_threads=2)
    assert len(results) == len(requests)
    assert stats["finished"] == len(requests) and stats["bytes_in_use"] == 0
    for k, (m, c, steps) in enumerate(requests):
        r, q = results[k]
        assert r["status"] == 0, r
        qs, st = solo(m, c, steps, 0.0 if steps else drop, precision)
        assert np.array_equal(q, qs), (k, np.abs(q - qs).max())
        assert r["iterations"] == st["iterations"] and r["t"] == st["t"]
        assert r["drag"] == st["drag"] and r["lift"] == st["lift"]
        assert r["done_reason"] == (2 if steps else 3)
        assert r["submit_s"] <= r["admit_s"] <= r["finish_s"]
    assert stats["cell_updates"] == sum(results[k][0]["iterations"] * m.n_cells
                                        for k, (m, _, _) in enumerate(requests))


def test_admission_respects_the_device_budget(requests):
    one = max(E.batch_footprint([m], [c], "split") for m, c, _ in requests)
    results, stats, _ = serve(requests, "split", hbm_budget=int(1.5 * one), tick_ms=1.0)
    assert len(results) == len(requests) and all(r["status"] == 0 for r, _ in results.values())
    assert 0 < stats["bytes_peak"] <= int(1.5 * one)
    admits = sorted(r["admit_s"] for r, _ in results.values())
    assert admits[-1] > admits[0]  # later requests waited for memory


def test_failed_requests_are_reported(requests):
    m, c, _ = requests[0]
    bad = bump_cfg(0.5)
    bad.n_boundaries = 2  # the Wall tag has no condition
    sv = E.EbbServer("split")
    i_bad = sv.submit(m, bad, 10)
    i_ok = sv.submit(m, c, 10)
    got = {}
    for _ in range(10000):
        a, w = sv.tick()
        for r in sv.results():
            got[r["id"]] = r
        if len(got) == 2 and a == 0 and w == 0:
            break
    assert got[i_bad]["status"] == 5 and "Wall" in got[i_bad]["msg"]
    assert got[i_ok]["status"] == 0 and got[i_ok]["iterations"] == 10
    with pytest.raises(E.EbbError):
        sv.take_state(i_bad)
    sv.close()


def _beyond_fp32():
    """A bump channel at density 1e-30 with the Rusanov flux: its averaged density
    sqrt(rhoL rhoR) needs the product 1e-60, below the FP32 range, so the split path's
    flux is NaN at the first step, while the FP64 solve is the density-scaled copy of
    an ordinary Mach 0.5 flow."""
    m = meshgen.bump_channel(3000, h=0.05, seed=5).to_solver_mesh()
    return m, bump_cfg(0.5, flux="rusanovFlux", rho=1e-30)


def test_split_error_escalates_to_fp64():
    m, c = _beyond_fp32()
    steps = 40
    s = E.UfvmSolver(m, c, "split")
    s.set_stop(0, t_end=c.t_end, max_steps=steps)
    with pytest.raises(E.EbbError) as ei:
        s.run(steps, records=False)
    assert ei.value.code in (8, 9)
    s.close()
    q64, st64 = solo(m, c, steps, 0.0, "fp64")
    for escalate in (0, 1):
        sv = E.EbbServer("split", escalate=escalate, tick_ms=2.0)
        rid = sv.submit(m, c, steps)
        got = None
        for _ in range(100000):
            a, w = sv.tick()
            for r in sv.results():
                got = r
            if got is not None and a == 0 and w == 0:
                break
        if escalate:
            assert got["status"] == 0 and got["escalated"] == 1 and got["precision"] == 0
            assert got["iterations"] == steps
            assert np.array_equal(sv.take_state(rid), q64)
            assert sv.stats()["escalations"] == 1
        else:
            assert got["status"] in (8, 9) and got["escalated"] == 0 and got["precision"] == 1
        sv.close()


def _serve_all(reqs, precision="split", **opts):
    """Submit every (mesh, cfg, max_steps, resid_drop) at once; run to completion."""
    sv = E.EbbServer(precision, **opts)
    ids = {sv.submit(m, c, n, d): k for k, (m, c, n, d) in enumerate(reqs)}
    out = {}
    for _ in range(1000000):
        a, w = sv.tick()
        for r in sv.results():
            out[ids[r["id"]]] = (r, sv.take_state(r["id"]))
        if len(out) == len(reqs) and a == 0 and w == 0:
            break
    sv.close()
    return out


def test_stalled_split_solve_finishes_in_fp64():
    """A split solve asked for a 1e-8 density-residual drop levels off at the FP32
    rounding of its increments; the server continues it in plain FP64 from its state
    (same id, iteration count, time and first-iteration residual) and retires it at the
    drop.  The result is the same served alone and in a mix with other requests."""
    m = meshgen.bump_channel(1500, h=0.05, seed=11).to_solver_mesh()
    c = bump_cfg(0.5, flux="rusanovFlux")
    drop, cap = 1e-8, 200000
    alone = _serve_all([(m, c, cap, drop)], tick_ms=2.0)
    r, q = alone[0]
    assert r["status"] == 0 and r["done_reason"] == 3, r
    assert r["escalated"] == 2 and r["precision"] == 0
    assert 0 < r["split_iterations"] < r["iterations"] < cap
    assert r["resid"][0] <= drop * r["resid_first"]
    assert r["submit_s"] <= r["admit_s"] <= r["finish_s"]
    others = [(meshgen.bump_channel(900, h=0.08, seed=12).to_solver_mesh(), bump_cfg(0.6, flux="rusanovFlux"), 300, 0.0),
              (meshgen.bump_channel(2000, h=0.03, seed=13).to_solver_mesh(), bump_cfg(0.4, flux="rusanovFlux"), 0, 1e-3)]
    mix = _serve_all(others[:1] + [(m, c, cap, drop)] + others[1:], tick_ms=2.0, max_batch=2)
    r2, q2 = mix[1]
    assert np.array_equal(q2, q)
    for f in ("iterations", "split_iterations", "t", "drag", "lift", "done_reason", "escalated"):
        assert r2[f] == r[f], f
    assert mix[0][0]["done_reason"] == 2 and mix[2][0]["done_reason"] == 3


def test_stalled_split_solve_finishes_in_df():
    """The same stalled split solve with the double-float form as the finishing form:
    the split phase is the same (same split iterations), the continuation retires at the
    drop in double-float, and its converged forces agree with the FP64-finished solve's.
    A solve served in double-float from the start reaches the drop without finishing."""
    m = meshgen.bump_channel(1500, h=0.05, seed=11).to_solver_mesh()
    c = bump_cfg(0.5, flux="rusanovFlux")
    drop, cap = 1e-8, 200000
    r64, q64 = _serve_all([(m, c, cap, drop)], tick_ms=2.0)[0]
    rdf, qdf = _serve_all([(m, c, cap, drop)], tick_ms=2.0, finish_precision="df")[0]
    assert rdf["status"] == 0 and rdf["done_reason"] == 3, rdf
    assert rdf["escalated"] == 2 and rdf["precision"] == 2
    assert rdf["split_iterations"] == r64["split_iterations"]
    assert rdf["resid"][0] <= drop * rdf["resid_first"]
    assert abs(rdf["drag"] - r64["drag"]) <= 1e-6 * abs(r64["drag"])
    assert np.abs(qdf - q64).max() <= 1e-6 * np.abs(q64).max()
    r, q = _serve_all([(m, c, cap, drop)], precision="df", tick_ms=2.0)[0]
    assert r["status"] == 0 and r["done_reason"] == 3 and r["escalated"] == 0 and r["precision"] == 2, r
    assert r["split_iterations"] == 0 and r["iterations"] < cap
    assert abs(r["drag"] - r64["drag"]) <= 1e-6 * abs(r64["drag"])
