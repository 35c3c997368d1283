"""Freestream preservation: a uniform state with far-field (fullState) boundaries is a
discrete steady state.  The split path subtracts each cell's own physical-flux edge
sum from its residual, so the state must not move at all (bit for bit), on triangles
and on mixed quads, pentagons and a hexagon, with either flux and the limiter on;
plain FP64 keeps it to rounding."""
import json

import numpy as np
import pytest

import ebbcfd_gb300 as E
from ebbcfd_gb300 import meshgen

pytestmark = pytest.mark.gpu


def far_field_cfg(flux, integrator):
    q = [0.63, 17.0, 1, 1.3]  # Mach 0.63 at 17 degrees: both velocity components nonzero
    return E.load_config(json.dumps({
        "mesh": "m.msh", "dt": 1e-4, "tEnd": 1000.0, "flux": flux, "saveIter": -1, "plotIter": -1,
        "forceBoundary": "Freestream", "initialConditions": q, "integrator": integrator, "CFL": 0.5,
        "boudaryConditions": [{"tag": "Freestream", "type": "fullState", "q": q}]}))


@pytest.mark.parametrize("flux,integrator", [("roeFlux", "RK2"), ("rusanovFlux", "RK4"), ("roeFlux", "RK2_TVD")])
@pytest.mark.parametrize("mesh", ["quads", "polygons"])
def test_uniform_flow_stays_uniform(flux, integrator, mesh):
    m = (meshgen.uniform_quads(24) if mesh == "quads" else meshgen.hanging_quads(16)).to_solver_mesh()
    cfg = far_field_cfg(flux, integrator)
    for precision in ("split", "fp64"):
        s = E.UfvmSolver(m, cfg, precision)
        q0 = s.state
        s.run(60, records=False)
        q = s.state
        if precision == "split":
            assert np.array_equal(q, q0), np.abs(q - q0).max()
        else:
            assert np.abs(q - q0).max() <= 1e-14 * np.abs(q0).max()
        s.close()
