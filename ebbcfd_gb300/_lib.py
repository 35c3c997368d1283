"""ctypes binding of include/ebb_gb300.h (the library's C ABI).

The shared library is built in-tree (ebbcfd_gb300/_build/libebbgb300.so).  Loading
fails loudly if it is missing: there is no CPU fallback for the solver.
"""
import ctypes as C
import os

from . import build as _build

MAX_BC = 32
FLUX_NOALLOC_MAX = 32768
MAX_FORCE = 8
TAG_LEN = 64
PATH_LEN = 1024

STATUS = {
    0: "EBB_OK", 1: "EBB_ERR_ARG", 2: "EBB_ERR_IO", 3: "EBB_ERR_FORMAT", 4: "EBB_ERR_MESH", 5: "EBB_ERR_CONFIG",
    6: "EBB_ERR_CUDA", 7: "EBB_ERR_OOM", 8: "EBB_ERR_NAN_EDGE", 9: "EBB_ERR_NAN_CELL", 10: "EBB_ERR_NO_DEVICE",
    11: "EBB_ERR_BC", 12: "EBB_ERR_LIMIT",
}


class Boundary(C.Structure):
    _fields_ = [("tag", C.c_char * TAG_LEN), ("type", C.c_int32), ("n_data", C.c_int32), ("data", C.c_double * 8)]


class Config(C.Structure):
    _fields_ = [
        ("mesh_file", C.c_char * PATH_LEN),
        ("dt", C.c_double),
        ("dynamic_dt", C.c_int32),
        ("t_end", C.c_double),
        ("flux", C.c_int32),
        ("save_iter", C.c_int64),
        ("plot_iter", C.c_int64),
        ("n_force", C.c_int32),
        ("force_boundary", (C.c_char * TAG_LEN) * MAX_FORCE),
        ("integrator", C.c_int32),
        ("limited", C.c_int32),
        ("lp_thresh", C.c_double),
        ("order", C.c_int64),
        ("cfl", C.c_double),
        ("ic", C.c_double * 4),
        ("n_boundaries", C.c_int32),
        ("boundaries", Boundary * MAX_BC),
        ("local_timestep", C.c_int32),
        ("multistage_limiting", C.c_int32),
        ("cfl_adjust", C.c_int32),
        ("viscosity", C.c_int32),
        ("pr", C.c_double),
        ("r_gas", C.c_double),
        ("gamma", C.c_double),
        ("mu", C.c_double),
        ("re", C.c_double),
        ("l_ref", C.c_double),
        ("mms", C.c_int32),
    ]


class MeshInfo(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("n_cells", C.c_int64), ("n_ghost", C.c_int64), ("n_edges", C.c_int64),
                ("n_int_edges", C.c_int64), ("n_tags", C.c_int32), ("max_edges", C.c_int32),
                ("face_slots", C.c_int64)]


class StepRecord(C.Structure):
    _fields_ = [("t", C.c_double), ("drag", C.c_double), ("lift", C.c_double), ("resid", C.c_double * 4),
                ("rmax", C.c_double), ("dt", C.c_double), ("cfl", C.c_double)]


class InstanceStatus(C.Structure):
    _fields_ = [("cell_offset", C.c_int64), ("n_cells", C.c_int64), ("iterations", C.c_int64),
                ("t", C.c_double), ("dt", C.c_double), ("cfl", C.c_double), ("done", C.c_int32),
                ("status", C.c_int32), ("err_index", C.c_int64), ("drag", C.c_double), ("lift", C.c_double),
                ("resid", C.c_double * 4), ("rmax", C.c_double), ("resid_first", C.c_double)]


class ServerOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("max_arenas", C.c_int32), ("max_batch", C.c_int32),
                ("build_threads", C.c_int32), ("tick_ms", C.c_double), ("size_ratio", C.c_double),
                ("arena_cells", C.c_int64), ("hbm_budget", C.c_uint64), ("escalate", C.c_int32),
                ("finish_fp64", C.c_int32), ("stall_steps", C.c_int32), ("finish_precision", C.c_int32)]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("done_reason", C.c_int32), ("err_index", C.c_int64),
                ("n_cells", C.c_int64), ("iterations", C.c_int64), ("t", C.c_double), ("drag", C.c_double),
                ("lift", C.c_double), ("resid", C.c_double * 4), ("resid_first", C.c_double),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double),
                ("precision", C.c_int32), ("escalated", C.c_int32), ("split_iterations", C.c_int64),
                ("msg", C.c_char * 96)]


class ServerStats(C.Structure):
    _fields_ = [("bytes_in_use", C.c_uint64), ("bytes_peak", C.c_uint64), ("arenas", C.c_int32),
                ("waiting", C.c_int32), ("building", C.c_int32), ("reserved", C.c_int32),
                ("submitted", C.c_int64), ("finished", C.c_int64), ("cell_updates", C.c_int64),
                ("escalations", C.c_int64)]


# every function the header declares, with its signature
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p
_cp = C.c_char_p
SIGNATURES = {
    "ebb_abi_version": (C.c_int, []),
    "ebb_struct_sizes": (C.c_int, [C.POINTER(C.c_size_t)] * 3),
    "ebb_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "ebb_set_device": (C.c_int, [C.c_int]),
    "ebb_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_vp)]),
    "ebb_host_free": (C.c_int, [_vp]),
    "ebb_config_defaults": (None, [C.POINTER(Config)]),
    "ebb_config_parse": (C.c_int, [_cp, C.POINTER(Config), _cp, C.c_size_t]),
    "ebb_mesh_import": (C.c_int, [_cp, C.POINTER(_vp), _cp, C.c_size_t]),
    "ebb_mesh_from_arrays": (C.c_int, [C.c_int64, _dp, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                       C.c_int64, C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int64), _cp,
                                       C.POINTER(_vp), _cp, C.c_size_t]),
    "ebb_mesh_get_info": (C.c_int, [_vp, C.POINTER(MeshInfo)]),
    "ebb_mesh_get_tag": (C.c_int, [_vp, C.c_int32, _cp, C.c_size_t]),
    "ebb_mesh_centroids": (C.c_int, [_vp, _dp]),
    "ebb_mesh_edges": (C.c_int, [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _dp, _dp, _dp]),
    "ebb_mesh_free": (None, [_vp]),
    "ebb_solver_create": (C.c_int, [_vp, C.POINTER(Config), C.c_int32, C.POINTER(_vp), _cp, C.c_size_t]),
    "ebb_solver_destroy": (None, [_vp]),
    "ebb_last_error": (C.c_int, [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int64), _cp, C.c_size_t]),
    "ebb_set_state": (C.c_int, [_vp, _dp]),
    "ebb_get_state": (C.c_int, [_vp, _dp]),
    "ebb_get_time": (C.c_int, [_vp, _dp, _dp, C.POINTER(C.c_int64)]),
    "ebb_set_time": (C.c_int, [_vp, C.c_double, C.c_double]),
    "ebb_residual": (C.c_int, [_vp, _dp, _dp, _dp, _dp, C.c_int32, C.c_int32]),
    "ebb_residual_device": (C.c_int, [_vp, _vp, _vp, _dp, _dp, C.c_int32, C.c_int32]),
    "ebb_step": (C.c_int, [_vp, _dp, _dp]),
    "ebb_run": (C.c_int, [_vp, C.c_int64, C.POINTER(StepRecord), C.POINTER(C.c_int64)]),
    "ebb_get_face_states": (C.c_int, [_vp, _dp]),
    "ebb_get_edge_fluxes": (C.c_int, [_vp, _dp]),
    "ebb_run_timed": (C.c_int, [_vp, C.c_int64, C.POINTER(C.c_int64), _dp]),
    "ebb_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "ebb_profile_kernels": (C.c_int, [_vp, C.c_int32, _dp]),
    "ebb_flux": (C.c_int, [C.c_int32, C.c_int64, _dp, _dp, _dp, _dp, _dp]),
    "ebb_flux_noalloc": (C.c_int, [C.c_int32, C.c_int64, _dp, _dp, _dp, _dp, _dp]),
    "ebb_batch_create": (C.c_int, [C.c_int32, C.POINTER(_vp), C.POINTER(Config), C.c_int32, C.POINTER(_vp), _cp,
                                   C.c_size_t]),
    "ebb_batch_size": (C.c_int, [_vp, C.POINTER(C.c_int32)]),
    "ebb_batch_status": (C.c_int, [_vp, C.c_int32, C.c_int32, C.POINTER(InstanceStatus)]),
    "ebb_batch_set_stop": (C.c_int, [_vp, C.c_int32, C.c_double, C.c_int64, C.c_double]),
    "ebb_batch_get_state": (C.c_int, [_vp, C.c_int32, _dp]),
    "ebb_batch_set_state": (C.c_int, [_vp, C.c_int32, _dp]),
    "ebb_launch_steps": (C.c_int, [_vp, C.c_int64]),
    "ebb_sync": (C.c_int, [_vp]),
    "ebb_batch_footprint": (C.c_int, [C.c_int32, C.POINTER(_vp), C.POINTER(Config), C.c_int32,
                                      C.POINTER(C.c_size_t), _cp, C.c_size_t]),
    "ebb_server_options_defaults": (None, [C.POINTER(ServerOptions)]),
    "ebb_server_create": (C.c_int, [C.POINTER(ServerOptions), C.POINTER(_vp), _cp, C.c_size_t]),
    "ebb_server_submit": (C.c_int, [_vp, _vp, C.POINTER(Config), C.c_int64, C.c_double, C.POINTER(C.c_int64)]),
    "ebb_server_tick": (C.c_int, [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ebb_server_results": (C.c_int, [_vp, C.POINTER(RequestResult), C.c_int32, C.POINTER(C.c_int32)]),
    "ebb_server_take_state": (C.c_int, [_vp, C.c_int64, _dp]),
    "ebb_server_stats_get": (C.c_int, [_vp, C.POINTER(ServerStats)]),
    "ebb_server_destroy": (None, [_vp]),
    "ebb_save_solution": (C.c_int, [_vp, _cp, C.c_double, C.c_double]),
    "ebb_load_solution": (C.c_int, [_vp, _cp]),
    "ebb_load_solution_parts": (C.c_int, [_vp, C.c_int32, C.POINTER(_cp)]),
    "ebb_reconstruct": (C.c_int, [_vp, _vp, _cp, _cp, C.c_double, C.c_double, _dp, C.POINTER(C.c_int64)]),
}

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load the shared library (building it first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("ebbcfd_gb300 native library not found at %s; run ebbcfd_gb300/build.py" % _build.LIB)
    L = C.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L
