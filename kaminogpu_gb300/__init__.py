"""GB300-native Kamino spherical fluid step (sm_103a CUDA kernels behind a C ABI).

The compute path is libkamino_gb300.so (csrc/); this package is the host-side
mirror of the reference's solver interface used by the tests and benchmarks.
"""
from . import _lib
from ._lib import (ERR_BUDGET, ERR_INVALID, ERR_NOT_READY, FRAME_GRID, FRAME_PARTICLES, F_HONOR_STEP_DT,
                   F_PARTICLE_RK2, F_POLE_SIGN_FLIP, F_REFERENCE_ROUNDING, OK, PARTICLES, PRESSURE, THICKNESS, U_PHI, U_THETA,
                   KaminoConfig, KaminoError, check, lib)
from .solver import (Kamino, KaminoSolver, default_config, read_ppm, frame_steps, make_initial_state, parse_config,
                     particle_count)

LIB_PATH = _lib.LIB_PATH
