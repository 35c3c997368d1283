"""Double-float precision form (EBB_PREC_DF) against the FP64 oracle, through the C ABI.

The df form evaluates faces, fluxes, gradients and limiters on pairs of FP32 numbers
(~46 significant bits) and keeps the FP64 solution update of the plain path, so its
results differ from the reference's FP64 arithmetic only in the last ~7 bits of each
operation: one residual evaluation within 3e-11 of the oracle's (relative to each
component's largest magnitude; measured: at most 1.03e-11, on a nearly uniform inflow
whose residuals are flux differences cancelling to ~1e-13 of the fluxes), the state
after 100 steps within 1e-8 (measured: at most 1.6e-9, in the cross-stream momentum
of the inviscid plate, a component whose values are differences of nearly equal
fluxes), the time and time-step columns within 1e-9 (the step follows the state's
wave speeds: measured 2e-10), forces and residual history within 1e-8; where the
oracle stops (a NaN flux, an inflow without a Mach root) the df path stops the same
way.
"""
import numpy as np
import pytest

import ebbcfd_gb300 as E
from tests.cases import all_cases, case
from tests.test_gpu_parity import NO_PERTURB, perturbed, rel_err

pytestmark = pytest.mark.gpu

NAMES = [c.name for c in all_cases()]
DF_RES_TOL = 3e-11
DF_STATE_TOL = 1e-8
DF_HIST_TOL = 1e-8


def df_solver(c):
    cfg = E.load_config(c.text)
    cfg.mms = c.mms
    return E.UfvmSolver(c.product_mesh(), cfg, "df")


@pytest.mark.parametrize("name", NAMES)
def test_df_residual_one_stage(name):
    c = case(name)
    _, om = c.build()
    s = df_solver(c)
    q = om.state() if name in NO_PERTURB else perturbed(om.state())
    for limit in (True, False):
        try:
            Ro, dto, rmo = om.residual(q, limit=limit)
        except RuntimeError as eo:
            with pytest.raises(E.EbbError) as eg:
                s.ufvm_solver(q, limit=limit)
            assert ("status %d" % eg.value.code) in str(eo)
            continue
        Rd, dtd, rmd = s.ufvm_solver(q, limit=limit)
        assert rel_err(Rd, Ro) <= DF_RES_TOL, (name, limit, rel_err(Rd, Ro))
        assert abs(dtd - dto) <= 1e-12 * abs(dto) and abs(rmd - rmo) <= 1e-11 * abs(rmo)
        assert rel_err(s.edge_fluxes(), om.edge_fluxes()) <= DF_RES_TOL
    s.close()


@pytest.mark.parametrize("name", NAMES)
def test_df_hundred_steps(name):
    c = case(name)
    _, om = c.build()
    s = df_solver(c)
    n = 100
    try:
        rec_o = om.run(n)
    except RuntimeError as eo:
        with pytest.raises(E.EbbError) as eg:
            s.run(n)
        assert ("status %d" % eg.value.code) in str(eo)
        return
    rec_d = s.run(n)
    assert len(rec_d) == n
    assert rel_err(s.state, om.state()) <= DF_STATE_TOL, rel_err(s.state, om.state())
    assert rel_err(rec_d[:, [0, 8]], rec_o[:, [0, 8]]) <= 1e-9
    # Each residual column is normalised by the sum of its state component over the
    # cells (app/solver.d).  Density and energy are positive, so their sums never
    # cancel; a momentum sum that crosses zero during the run (the oracle's column
    # changes sign: the cross-stream momentum of a flow along the x axis) makes the
    # column's value a ratio to a cancelled sum, dominated by the cancellation in the
    # oracle as in any other arithmetic, and that column is not compared.
    cols = [3, 6] + [k for k in (4, 5) if np.all(rec_o[:, k] > 0) or np.all(rec_o[:, k] < 0)]
    assert rel_err(rec_d[:, cols], rec_o[:, cols]) <= DF_HIST_TOL
    fscale = max(np.abs(rec_o[:, 1:3]).max(), 1.0)
    assert np.abs(rec_d[:, 1:3] - rec_o[:, 1:3]).max() <= DF_HIST_TOL * fscale
    s.close()


def test_df_batch_instances_equal_single_solves():
    """A batched arena in the df form: every instance bitwise its own single solve."""
    cs = [case("wedge_rusanov"), case("bump_roe_tvd")]
    import json
    # one arena needs one flux and integrator: run both meshes with the wedge's physics
    text = cs[0].text
    meshes = [c.product_mesh() for c in cs]
    cfgs = [E.load_config(text) for _ in cs]
    d = json.loads(cs[1].text)
    cfgs[1] = E.load_config(json.dumps(dict(json.loads(text), boudaryConditions=[
        {"tag": b["tag"], "type": "fullState" if b["type"] == "fullState" else "inviscidWall", "q": [2.5, 0, 1, 1]}
        for b in d["boudaryConditions"]])))
    b = E.UfvmBatch(meshes, cfgs, "df")
    b.set_stop(-1, max_steps=40)
    b.run(10 ** 6, records=False)
    for k, (m, cf) in enumerate(zip(meshes, cfgs)):
        s = E.UfvmSolver(m, cf, "df")
        s.run(40, records=False)
        assert np.array_equal(b.instance_state(k), s.state), k
        s.close()
    b.close()
