"""GB300-native explicit second-order unstructured finite-volume update (EbbCFD's hot path).

The compute path is hand-written CUDA for sm_103a behind the C ABI of
include/ebb_gb300.h; this package holds the build script, the ctypes binding and a
Python mirror of the reference's operator interface.
"""
from .solver import (CellException, EbbError, EbbServer, EdgeException, Mesh, UfvmBatch, UfvmSolver, batch_footprint,
                     default_config, import_mesh, load_config, roe_flux, rusanov_flux, set_boundaries,
                     set_force_boundary)

__all__ = ["CellException", "EbbError", "EbbServer", "EdgeException", "Mesh", "UfvmBatch", "UfvmSolver", "batch_footprint",
           "default_config", "import_mesh", "load_config", "roe_flux", "rusanov_flux", "set_boundaries",
           "set_force_boundary"]
