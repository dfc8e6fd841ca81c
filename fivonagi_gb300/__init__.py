"""fivonagi_gb300 -- FiVoNAGI's time-step hot path on GB300 (sm_103a).

The product is libfivonagi.so (fivonagi_gb300/csrc, C ABI in
include/fivonagi.h); this package declares its types (_abi), mirrors the
reference's driver (solver.Simulation) and builds the library (build).
"""
from ._abi import (APP_NAMES, FV_APP_FOCUSED_BEAM, FV_APP_HIFU_BEAM, FV_APP_PHASED_ARRAY,
                   FV_APP_PLANE_WAVE, FV_APP_TAYLOR_ANGLE_XY, FV_STAGE_BOUNDARY, FV_STAGE_SOURCE,
                   FV_STAGE_SWEEP_X, FV_STAGE_SWEEP_Y, FvError, FvParams, FvRunStats,
                   default_params, load_library)
from .solver import Batch, Simulation

__all__ = [
    "APP_NAMES", "FV_APP_FOCUSED_BEAM", "FV_APP_HIFU_BEAM", "FV_APP_PHASED_ARRAY", "FV_APP_PLANE_WAVE",
    "FV_APP_TAYLOR_ANGLE_XY", "FV_STAGE_BOUNDARY", "FV_STAGE_SOURCE", "FV_STAGE_SWEEP_X",
    "FV_STAGE_SWEEP_Y", "Batch", "FvError", "FvParams", "FvRunStats", "Simulation", "default_params",
    "load_library",
]
