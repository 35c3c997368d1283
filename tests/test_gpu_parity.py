"""CUDA path vs the oracle, through the C ABI (GPU).

Bar: plain FP64 GPU residual within 1e-12 relative per cell after one
stage, state within 1e-9 relative after 100 steps.  The FP64 kernels keep the
reference's operation order without fused multiply-adds, so most cases agree
bitwise; the constant-pressure ghost state uses CUDA's pow(), which may differ from
the host libm's in the last place, so those cases are held to the stated tolerance.
"""
import numpy as np
import pytest

import ebbcfd_gb300 as E
from oracle import ref
from tests.cases import all_cases, case

pytestmark = pytest.mark.gpu

NAMES = [c.name for c in all_cases()]
USES_POW = {"flatplate_ns", "plate_ns_rk4", "bump_tpinflow_roe"}  # constP / tpInflow ghosts (solve.d:570-689)
# cases evaluated on their initial state: a perturbed inlet state leaves the tpInflow
# Mach quadratic (solve.d:641-669) without a non-negative root
NO_PERTURB = {"bump_tpinflow_roe"}
RES_TOL = 1e-12
STATE_TOL = 1e-9


def perturbed(q, seed=0):
    rng = np.random.default_rng(seed)
    q = q.copy()
    n = len(q)
    rho = q[:, 0] * (1 + 0.05 * rng.uniform(-1, 1, n))
    u = q[:, 1] / q[:, 0] + 0.05 * rng.uniform(-1, 1, n)
    v = q[:, 2] / q[:, 0] + 0.05 * rng.uniform(-1, 1, n)
    p = 0.4 * (q[:, 3] - 0.5 * q[:, 0] * ((q[:, 1] / q[:, 0]) ** 2 + (q[:, 2] / q[:, 0]) ** 2))
    p = p * (1 + 0.05 * rng.uniform(-1, 1, n))
    out = np.column_stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)])
    return out


def rel_err(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return (np.abs(a - b).max(axis=0) / scale).max()


@pytest.mark.parametrize("name", NAMES)
def test_residual_one_stage(name):
    sol, om = case(name).build()
    q = om.state() if name in NO_PERTURB else perturbed(om.state())
    for limit in (True, False):
        try:
            Ro, dto, rmo = om.residual(q, limit=limit)
        except RuntimeError as eo:
            # the reference stops (e.g. the unlimited reconstruction next to the tpInflow
            # ghost state gives a NaN flux): the GPU path stops the same way
            with pytest.raises(E.EbbError) as eg:
                sol.ufvm_solver(q, limit=limit)
            assert ("status %d" % eg.value.code) in str(eo) and ("index %d" % eg.value.index) in str(eo)
            assert limit is False or name not in NO_PERTURB
            continue
        Rg, dtg, rmg = sol.ufvm_solver(q, limit=limit)
        assert rel_err(Rg, Ro) <= RES_TOL, (name, limit, rel_err(Rg, Ro))
        assert abs(dtg - dto) <= 1e-14 * abs(dto)
        assert abs(rmg - rmo) <= 1e-12 * abs(rmo)
        assert rel_err(sol.face_states(), om.face_states()) <= RES_TOL
        # len * flux per edge (reference edge order), the terms of the residual and forces
        fg, fo = sol.edge_fluxes(), om.edge_fluxes()
        assert rel_err(fg, fo) <= RES_TOL, (name, limit, rel_err(fg, fo))
        if name not in USES_POW:
            assert np.array_equal(Rg, Ro), (name, limit, np.abs(Rg - Ro).max())
            assert dtg == dto and rmg == rmo
            assert np.array_equal(fg, fo)
    # determinism: same inputs, same bits
    Rg2, _, _ = sol.ufvm_solver(q, limit=True)
    Rg1, _, _ = sol.ufvm_solver(q, limit=True)
    assert np.array_equal(Rg1, Rg2)


@pytest.mark.parametrize("name", NAMES)
def test_hundred_steps(name):
    c = case(name)
    sol, om = c.build()
    nsteps = 100
    err_o = err_g = None
    try:
        rec_o = om.run(nsteps)
    except RuntimeError as e:
        err_o = str(e)
        rec_o = None
    try:
        rec_g = sol.run(nsteps)
    except E.EbbError as e:
        err_g = e
        rec_g = None
    if err_o or err_g:
        # both paths must fail the same way at the same place
        assert err_o and err_g, (err_o, err_g)
        assert ("status %d" % err_g.code) in err_o and ("index %d" % err_g.index) in err_o
        return
    assert len(rec_g) == len(rec_o) == nsteps
    qo, qg = om.state(), sol.state
    assert rel_err(qg, qo) <= STATE_TOL, rel_err(qg, qo)
    # t, dt, Rmax columns; RMS residuals and forces come from differently ordered sums
    assert rel_err(rec_g[:, [0, 8]], rec_o[:, [0, 8]]) <= 1e-12
    assert rel_err(rec_g[:, 7:8], rec_o[:, 7:8]) <= 1e-11
    assert rel_err(rec_g[:, 3:7], rec_o[:, 3:7]) <= 1e-9
    # forces: sums over the tagged wall edges in a different order; near-zero net
    # forces (symmetric walls) are compared against the size of the summed terms
    fscale = max(np.abs(rec_o[:, 1:3]).max(), 1.0)
    assert np.abs(rec_g[:, 1:3] - rec_o[:, 1:3]).max() <= 1e-9 * fscale
    if c.name not in USES_POW:
        assert np.array_equal(qg, qo), np.abs(qg - qo).max()


@pytest.mark.parametrize("integrator", ["Euler", "RK2", "RK2_TVD", "RK4"])
def test_integrator_step_seam(integrator):
    """One integrator.step!solver call (integrators.d) with an explicit dt and Rmax."""
    sol, om = case("mms_tri_limited").build(integrator=integrator)
    dt0 = 2e-4
    dto = np.array([dt0])
    rmo = np.array([0.0])
    st = ref.lib().o_step(om.h, ref._dp(dto), ref._dp(rmo))
    assert st == 0
    dtg, rmg = sol.step(dt0, 0.0)
    assert dtg == dto[0] and rmg == rmo[0]
    assert np.array_equal(sol.state, om.state())


def test_roe_known_answers_on_device(golden_dir):
    import json
    import os
    kat = json.load(open(os.path.join(golden_dir, "roe_kat.json")))
    for c in kat["cases"]:
        q, _, _ = ref.mms_eval(1, [c["p1"], c["p2"]])
        F, s = E.roe_flux(q[0], q[1], c["n"])
        assert np.abs(F[0] - np.array(c["F"])).max() <= 5e-16


@pytest.mark.parametrize("kind", [0, 1])
def test_flux_seam_bitwise(kind):
    rng = np.random.default_rng(kind)
    n = 20000
    rho = rng.uniform(0.2, 3, (n, 2))
    u = rng.uniform(-3, 3, (n, 2))
    v = rng.uniform(-3, 3, (n, 2))
    p = rng.uniform(0.1, 5, (n, 2))
    q = np.stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)], axis=-1)
    th = rng.uniform(0, 2 * np.pi, n)
    nrm = np.column_stack([np.cos(th), np.sin(th)])
    Fo, so = ref.flux_batch(kind, q[:, 0], q[:, 1], nrm)
    Fg, sg = (E.roe_flux if kind == 1 else E.rusanov_flux)(q[:, 0], q[:, 1], nrm)
    assert np.array_equal(Fg, Fo) and np.array_equal(sg, so)


def test_nan_state_reports_edge_like_reference():
    """A NaN in the state is caught as a NaN face flux with the reference's first edge id."""
    sol, om = case("bump_roe_tvd").build()
    q = om.state()
    q[17, 0] = np.nan
    with pytest.raises(RuntimeError) as eo:
        om.residual(q)
    with pytest.raises(E.EdgeException) as eg:
        sol.ufvm_solver(q)
    assert ("index %d" % eg.value.index) in str(eo.value)
    # the solver stays usable
    R, _, _ = sol.ufvm_solver(om.state())
    assert np.isfinite(R).all()


def test_save_load_roundtrip(tmp_path):
    sol, om = case("mms_tri_limited").build()
    sol.run(3)
    p = tmp_path / "s.esln"
    sol.save_solution(str(p))
    q = sol.state
    t, dt, _ = sol.time()
    sol2, _ = case("mms_tri_limited").build()
    sol2.load_solution(str(p))
    assert np.array_equal(sol2.state, q)
    t2, dt2, _ = sol2.time()
    assert (t2, dt2) == (t, dt)


def _write_esln_part(path, ids, q, t, dt, nedges):
    """.esln v2 holding only the cells `ids` (one rank's file of a partitioned run,
    io.d:68-161): global id, edge count, state, zero face states, then 4 CRC bytes."""
    import struct
    b = bytearray(struct.pack(">III", 0xEA98E1F5, 2, len(ids)) + struct.pack(">dd", t, dt) + struct.pack(">II", 4, 2))
    for i in ids:
        b += struct.pack(">IB", int(i), int(nedges[i])) + struct.pack(">4d", *q[i]) + bytes(32 * int(nedges[i]))
    b += bytes(4)
    open(path, "wb").write(bytes(b))


def test_load_solution_parts_places_cells_by_global_id(tmp_path):
    sol, om = case("mms_tri_limited").build()
    sol.run(3)
    q = sol.state
    t, dt, _ = sol.time()
    n = len(q)
    nedges = np.full(n, 3)
    rng = np.random.default_rng(0)
    perm = rng.permutation(n)
    parts = [perm[: n // 3], perm[n // 3:]]  # two "ranks", cells in arbitrary order
    paths = []
    for r, ids in enumerate(parts):
        p = tmp_path / ("save_0_%d.esln" % r)
        _write_esln_part(p, ids, q, t if r == 0 else 0.0, dt if r == 0 else 0.0, nedges)
        paths.append(str(p))
    sol2, _ = case("mms_tri_limited").build()
    sol2.load_solution_parts(paths)
    assert np.array_equal(sol2.state, q)
    assert sol2.time()[:2] == (t, dt)  # from the first file
    with pytest.raises(E.EbbError):  # one rank's file alone leaves cells uncovered
        sol2.load_solution_parts(paths[1:])


def test_tpinflow_case_drives_the_inflow_code():
    """The tpInflow parity case really runs the total-temperature/pressure inflow: its
    ghost states hold the solve.d:678-681 quirk (every value written into component 0,
    the others left at zero), so the inflow edges' fluxes differ from a freestream
    inflow's, on the GPU as in the oracle."""
    sol, om = case("bump_tpinflow_roe").build()
    q = om.state()
    Rg, _, _ = sol.ufvm_solver(q)
    Ro, _, _ = om.residual(q)
    assert rel_err(Rg, Ro) <= RES_TOL
    edges = sol.mesh.edges()
    inflow = edges["group"] == sol.mesh.tags.index("Inflow")
    fg, fo = sol.edge_fluxes(), om.edge_fluxes()
    assert inflow.sum() > 10 and rel_err(fg[inflow], fo[inflow]) <= RES_TOL
    # a uniform state and a freestream inflow would give zero net mass flux differences
    # along the inlet; the quirky ghost state does not
    assert np.abs(fg[inflow, 0]).max() > 1e-3
    # the quirky inflow drives the inlet cells away from a physical state: four steps
    # run, and the fifth stops at a boundary edge whose Mach quadratic has no
    # non-negative root (solve.d:662-669) -- on both paths, at the same edge
    sol, om = case("bump_tpinflow_roe").build()
    rec_o, rec_g = om.run(4), sol.run(4)
    assert len(rec_o) == len(rec_g) == 4
    assert rel_err(sol.state, om.state()) <= STATE_TOL
    with pytest.raises(RuntimeError) as eo:
        om.run(1)
    with pytest.raises(E.EbbError) as eg:
        sol.run(1)
    assert eg.value.code == 11  # EBB_ERR_BC
    assert ("status %d" % eg.value.code) in str(eo.value) and ("index %d" % eg.value.index) in str(eo.value)


def _cfl_case():
    """1024 quads on [0,1]^2, every boundary a Mach 1.2 freestream at 0 degrees, started
    from a Mach 1.2 stream at 5 degrees (Rusanov, limited, RK2, CFL 0.25, cflAdjust on):
    as the far field flushes the vertical momentum out, the sum of rho v falls towards
    zero faster than its increments, so the v-momentum RMS residual (app/solver.d:153-171)
    rises step after step for over 2000 steps and the CFL auto-adjust of
    app/solver.d:196-216 fires."""
    import json
    from ebbcfd_gb300 import meshgen
    from oracle import gmsh_ref
    g = meshgen.uniform_quads(32)
    text = json.dumps({"mesh": "sq.msh", "dt": 1e-4, "tEnd": 1e9, "flux": "rusanovFlux", "saveIter": -1,
                       "plotIter": -1, "forceBoundary": "Freestream", "integrator": "RK2", "limited": True,
                       "CFL": 0.25, "initialConditions": [1.2, 5, 1, 1],
                       "boudaryConditions": [{"tag": "Freestream", "type": "fullState", "q": [1.2, 0, 1, 1]}]})
    om = ref.OracleMesh(g.as_reader_dict(), gmsh_ref.load_config(text))
    sol = E.UfvmSolver(g.to_solver_mesh(), E.load_config(text))
    return sol, om


def _cfl_replay(rec):
    """Steps (0-based) at which app/solver.d:196-216's counter reaches 2000, replayed on a
    residual history (columns 3..6)."""
    last, inc, out = 0.0, 0, []
    for s, r in enumerate(rec):
        m = max(r[3:7])
        if last < m:
            inc += 1
        elif inc >= 1:
            inc -= 1
        if inc >= 2000:
            out.append(s)
            inc = 0
        last = m
    return out


def test_cfl_auto_adjust_after_2000_rising_steps():
    sol, om = _cfl_case()
    n = 4000
    rec_o = om.run(n)
    trig = _cfl_replay(rec_o)
    assert trig, "the case must make the CFL auto-adjust fire"
    c = ref.OCfg()
    ref.lib().o_get_cfg(om.h, c)
    assert c.CFL == 0.25 * 0.99 ** len(trig)
    rec_g = sol.run(n)
    assert len(rec_g) == n
    # the cfl column changes at the step the reference's counter reaches 2000
    changed = np.nonzero(rec_g[:, 9] != 0.25)[0]
    assert len(changed) and changed[0] == trig[0], (changed[:3], trig)
    assert rec_g[-1, 9] == c.CFL
    qo, qg = om.state(), sol.state
    assert rel_err(qg, qo) <= STATE_TOL
    assert np.array_equal(rec_g[:, [0, 8]], rec_o[:, [0, 8]])


def _fallback_state(om, seed=0, pf=0.2):
    """A Mach 2.5 wedge state with +-30% density and speed noise, random vertical
    velocity and 5-15% of the freestream pressure: the reconstructed pressure of many
    faces turns negative, so the per-direction minimum limiter of solve.d:996-1009
    (interior) and updateBoundaryEdge's lim[0] form (solve.d:306-318) take over."""
    q = om.state()
    n = len(q)
    rng = np.random.default_rng(seed)
    rho = q[:, 0] * (1 + 0.3 * rng.uniform(-1, 1, n))
    u = q[:, 1] / q[:, 0] * (1 + 0.3 * rng.uniform(-1, 1, n))
    v = 0.5 * rng.uniform(-1, 1, n)
    p0 = 0.4 * (q[:, 3] - 0.5 * q[:, 0] * ((q[:, 1] / q[:, 0]) ** 2 + (q[:, 2] / q[:, 0]) ** 2))
    p = p0 * pf * (1 + 0.5 * rng.uniform(-1, 1, n))
    return np.column_stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)])


def test_negative_pressure_fallback_interior_and_boundary():
    sol, om = case("wedge_rusanov").build()
    q = _fallback_state(om)
    Ro, dto, rmo = om.residual(q, limit=True)
    n_int, n_bnd = om.fallback_counts()
    assert n_int > 100 and n_bnd > 0, (n_int, n_bnd)
    Rg, dtg, rmg = sol.ufvm_solver(q, limit=True)
    assert np.array_equal(Rg, Ro) and dtg == dto and rmg == rmo
    assert np.array_equal(sol.face_states(), om.face_states())
    # lower pressures: faces still negative after the fallback give a NaN flux; both
    # paths stop at the same edge (the first in the reference's loop order)
    q2 = _fallback_state(om, pf=0.05)
    with pytest.raises(RuntimeError) as eo:
        om.residual(q2, limit=True)
    with pytest.raises(E.EbbError) as eg:
        sol.ufvm_solver(q2, limit=True)
    assert ("status %d" % eg.value.code) in str(eo.value) and ("index %d" % eg.value.index) in str(eo.value)


SPLIT_CASES = ["wedge_rusanov", "plate_ns_rk4", "mms_tri_limited"]
# split precision against the FP64 oracle after 100 steps (FP32 flux, gradient and
# limiter arithmetic): state per component relative to the component's largest
# magnitude, forces relative to the largest force, residual history relative
SPLIT_STATE_TOL = 2e-4
SPLIT_FORCE_TOL = 1e-4
SPLIT_RESID_TOL = 2e-2


@pytest.mark.parametrize("name", SPLIT_CASES)
def test_split_path_within_stated_tolerance_of_oracle_over_100_steps(name):
    c = case(name)
    _, om = c.build()
    cfg = E.load_config(c.text)
    cfg.mms = c.mms
    s32 = E.UfvmSolver(c.product_mesh(), cfg, "split")
    n = 100
    rec_o = om.run(n)
    rec_s = s32.run(n)
    assert len(rec_s) == n
    qo, qs = om.state(), s32.state
    err = rel_err(qs, qo)
    fscale = max(np.abs(rec_o[:, 1:3]).max(), 1e-300)
    ferr = np.abs(rec_s[:, 1:3] - rec_o[:, 1:3]).max() / fscale
    rerr = np.abs(rec_s[:, 3:7] / rec_o[:, 3:7] - 1).max()
    print(name, "state", err, "forces", ferr, "resid", rerr)
    assert err <= SPLIT_STATE_TOL, err
    assert ferr <= SPLIT_FORCE_TOL, ferr
    assert rerr <= SPLIT_RESID_TOL, rerr
    # same time levels: dt is computed in FP32 from FP32 wave speeds
    assert np.abs(rec_s[:, 0] - rec_o[:, 0]).max() <= 1e-5 * max(rec_o[-1, 0], 1e-300)
