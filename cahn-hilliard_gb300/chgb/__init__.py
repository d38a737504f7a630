"""chgb — GB300 (sm_103a, FP64) Cahn–Hilliard time-step engine, Python side.

The compute path is the CUDA library ``libchgb.so`` behind the C ABI in
include/chgb.h; this package only binds it (ctypes), builds its parameters
from the reference's TOML keys, and wraps it for PyTorch.
"""
from . import abi, config  # noqa: F401
from .sim import CahnHilliard  # noqa: F401,E402
