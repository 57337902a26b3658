"""GB300-native ideal-MHD solver step (MHDTurbulence hot path).

The compute path is libmhdgb.so (hand-written CUDA for sm_103a behind a C ABI, include/mhdgb.h);
this package holds its build script, the ctypes host mirror of the reference stage interface and
the seeded initial-condition generators.
"""
from . import ic  # noqa: F401
from ._lib import MhdgbError  # noqa: F401
from .ensemble import Ensemble, kh_ensemble_specs  # noqa: F401
from .solver import Solver  # noqa: F401

__all__ = ["Solver", "Ensemble", "kh_ensemble_specs", "MhdgbError", "ic"]
