"""Parity cases shared by the GPU tests and __graft_entry__.smoke(): each builds the
same mesh and config for the CUDA path (through the C ABI) and for the oracle."""
import json
import os

from ebbcfd_gb300 import meshgen
import ebbcfd_gb300 as E
from oracle import gmsh_ref, ref

HERE = os.path.dirname(os.path.abspath(__file__))
MESHES = os.path.join(HERE, "golden", "meshes")


def cfg_json(**kw):
    d = {"mesh": "m.msh", "dt": 1e-4, "tEnd": 1000.0, "flux": "roeFlux", "saveIter": -1, "plotIter": -1,
         "forceBoundary": "Wall", "initialConditions": [0.5, 0.0, 1.0, 1.0], "boudaryConditions": []}
    d.update(kw)
    return json.dumps(d)


class Case:
    def __init__(self, name, mesh_file=None, gen=None, text=None, mms=0):
        self.name = name
        self.mesh_file = mesh_file
        self.gen = gen
        self.text = text
        self.mms = mms

    def reader_mesh(self):
        if self.mesh_file:
            return gmsh_ref.parse_gmsh(os.path.join(MESHES, self.mesh_file))
        return self.gen().as_reader_dict()

    def product_mesh(self):
        if self.mesh_file:
            return E.import_mesh(os.path.join(MESHES, self.mesh_file))
        return self.gen().to_solver_mesh()

    def build(self, integrator=None):
        text = self.text
        if integrator:
            d = json.loads(text)
            d["integrator"] = integrator
            text = json.dumps(d)
        conf = gmsh_ref.load_config(text)
        om = ref.OracleMesh(self.reader_mesh(), conf, mms=self.mms)
        cfg = E.load_config(text)
        cfg.mms = self.mms
        sol = E.UfvmSolver(self.product_mesh(), cfg)
        return sol, om


def mms_text(name, **kw):
    d = json.loads(open(os.path.join(MESHES, name)).read())
    d.update(kw)
    return json.dumps(d)


def all_cases():
    fp = open(os.path.join(MESHES, "flatPlate_0.json")).read()
    fpd = json.loads(fp)
    fpd["flux"] = "rusanovFlux"
    fpd["limited"] = True
    fpd["viscosity"] = False
    fpd["boudaryConditions"][1]["type"] = "inviscidWall"
    fp_rus = json.dumps(fpd)
    wedge_bcs = [{"tag": "Inflow", "type": "fullState", "q": [2.5, 0, 1, 1]},
                 {"tag": "Top", "type": "fullState", "q": [2.5, 0, 1, 1]},
                 {"tag": "Symmetry", "type": "symmetry", "q": [2.5, 0, 1, 1]},
                 {"tag": "Ramp", "type": "inviscidWall", "q": [2.5, 0, 1, 1]},
                 {"tag": "Outflow", "type": "fullState", "q": [2.5, 0, 1, 1]}]
    bump_bcs = [{"tag": "Inflow", "type": "fullState", "q": [0.5, 0, 1, 1]},
                {"tag": "Outflow", "type": "fullState", "q": [0.5, 0, 1, 1]},
                {"tag": "Wall", "type": "inviscidWall", "q": [0.5, 0, 1, 1]}]
    plate_bcs = [{"tag": "Inflow", "type": "fullState", "q": [0.3, 0, 1, 1]},
                 {"tag": "Top", "type": "fullState", "q": [0.3, 0, 1, 1]},
                 {"tag": "Outflow", "type": "constP", "q": [7.936507936507937]},
                 {"tag": "Symmetry", "type": "symmetry", "q": [0.3, 0, 1, 1]},
                 {"tag": "Wall", "type": "viscidWall", "q": [0.3, 0, 1, 1]}]
    # total temperature / total pressure inflow (solve.d:625-689, flux solve.d:939) for a
    # Mach 0.5 stream with R = 1: T = p / rho = 1 / (1.4 * 0.25), Tt = T (1 + 0.2 M^2),
    # Pt = p (Tt / T)^3.5.  The inflow direction is 180 degrees: solve.d:641-647 dots it
    # with the boundary edge's outward normal, and only an inflow direction against that
    # normal (d = +1 at the left inlet) gives the quadratic a non-negative Mach root
    t_inf = 1.0 / (1.4 * 0.25)
    tp_bcs = [{"tag": "Inflow", "type": "tpInflow", "q": [t_inf * 1.05, t_inf * 1.05 ** 3.5, 180.0]},
              {"tag": "Outflow", "type": "fullState", "q": [0.5, 0, 1, 1]},
              {"tag": "Wall", "type": "inviscidWall", "q": [0.5, 0, 1, 1]}]
    sym_visc = dict(json.loads(fp))
    return [
        Case("mms_quads_lp", "ms_refine_3.msh", text=mms_text("ms_refine_3.json"), mms=1),
        Case("mms_tri_limited", "ms_refine_tri_2.msh", text=mms_text("ms_refine_3.json", lpThresh=-1), mms=1),
        Case("mms_tri_pert_lp", "ms_refine_tri_pert_1.msh", text=mms_text("ms_refine_3.json"), mms=1),
        Case("mms_ns_quads", "ms_refine_1.msh", text=mms_text("ms_refine_vs_0.json", limited=True), mms=1),
        Case("flatplate_ns", "flatPlate_0.msh", text=fp),
        Case("flatplate_rusanov_inviscid", "flatPlate_0.msh", text=fp_rus),
        Case("wedge_rusanov", gen=lambda: meshgen.wedge(6000, seed=0),
             text=cfg_json(flux="rusanovFlux", initialConditions=[2.5, 0, 1, 1], boudaryConditions=wedge_bcs,
                           forceBoundary="Ramp", CFL=0.4, integrator="RK2")),
        Case("bump_roe_tvd", gen=lambda: meshgen.bump_channel(3000, h=0.08),
             text=cfg_json(initialConditions=[0.5, 0, 1, 1], boudaryConditions=bump_bcs, integrator="RK2_TVD")),
        Case("plate_ns_rk4", gen=lambda: meshgen.flat_plate(8000, layer_top=0.01),
             text=cfg_json(initialConditions=[0.3, 0, 1, 1], boudaryConditions=plate_bcs, integrator="RK4",
                           viscosity=True, physicalConfig={"Pr": 0.72, "R": 1.0, "gamma": 1.4, "Re": 1e5, "L": 1.0},
                           CFL=0.8)),
        Case("sine_quads_tvd", gen=lambda: meshgen.uniform_quads(32),
             text=cfg_json(initialConditions=[0.5, 0, 1, 1], integrator="RK2_TVD",
                           boudaryConditions=[{"tag": "Freestream", "type": "dirichlet", "q": [0.5, 0, 1, 1]}],
                           CFL=0.5), mms=2),
        # pentagons and a hexagon (hanging nodes): the six-neighbour kernels
        Case("hanging_polygons_rk2", gen=lambda: meshgen.hanging_quads(16),
             text=cfg_json(initialConditions=[0.5, 0, 1, 1], integrator="RK2",
                           boudaryConditions=[{"tag": "Freestream", "type": "dirichlet", "q": [0.5, 0, 1, 1]}],
                           CFL=0.5), mms=2),
        Case("bump_tpinflow_roe", gen=lambda: meshgen.bump_channel(3000, h=0.05, seed=2),
             text=cfg_json(initialConditions=[0.5, 0, 1, 1], boudaryConditions=tp_bcs, integrator="RK2",
                           physicalConfig={"Pr": 0.72, "R": 1.0, "gamma": 1.4, "Re": 1000, "L": 1.0})),
        Case("order1_local_dt", "ms_refine_tri_1.msh",
             text=mms_text("ms_refine_3.json", order=1, localTimestep=True, lpThresh=-1), mms=1),
    ]


def case(name):
    for c in all_cases():
        if c.name == name:
            return c
    raise KeyError(name)
