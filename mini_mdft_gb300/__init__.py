"""mini_mdft_gb300 -- GB300 (sm_103a) implementation of Mini-MDFT's
excess-functional convolution hot path behind a C ABI
(include/mdft_gb300.h), with a Python mirror of the reference's operator API.
"""
from . import inputs  # noqa: F401
from .api import (  # noqa: F401
    MDFT_F32,
    MDFT_F64,
    MDFT_F64_DF,
    AngularGrid,
    Convolution,
    MdftError,
    OrientationProjectionMap,
    OrientationProjectionTransform,
    Server,
    Solver,
    SpatialGrid,
    get_delta_f,
    get_delta_rho,
    luc_read,
    luc_write,
    solute_vext,
    wait_timeouts,
    wait_selftest,
    grid_barrier_selftest,
)
from ._lib import LIB_PATH, lib  # noqa: F401
from .solvent import Solvents, check_mole_fractions, mole_fractions  # noqa: F401

