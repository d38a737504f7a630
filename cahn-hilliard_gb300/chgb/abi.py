"""ctypes view of the C ABI declared in include/chgb.h.

The structures mirror ``chgb_model_params`` / ``chgb_params`` field by field
(same order, same C types), so ctypes lays them out exactly as the C compiler
does.  ``load_library()`` loads the in-tree ``libchgb.so`` and fails loudly
when it is missing: there is no CPU fallback for the product path.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # cahn-hilliard_gb300/
REPO_ROOT = PKG_ROOT.parent
LIB_PATH = PKG_ROOT / "lib" / "libchgb.so"
HEADER_PATH = REPO_ROOT / "include" / "chgb.h"

CHGB_ABI_VERSION = 5
CHGB_MAX_SPECIES = 3

# status codes
CHGB_OK = 0
CHGB_ERR_INVALID = 1
CHGB_ERR_CUDA = 2
CHGB_ERR_NAN = 3
CHGB_ERR_UNSUPPORTED = 4
CHGB_ERR_ALLOC = 5
CHGB_ERR_TIMEOUT = 6

INTEGRATORS = {"euler": 0, "euler_mobility": 1, "pseudospectral": 2, "pseudospectral_mobility": 3}
MODELS = {"landau": 0, "simple_wertheim": 1, "saleh": 2}
MOBILITIES = {"constant": 0, "free_energy": 1, "regularised": 2, "gel": 3}
N_SPECIES = {"landau": 1, "simple_wertheim": 1, "saleh": 3}


class ModelParams(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("n_species", ctypes.c_int32),
        ("epsilon", ctypes.c_double),
        ("valence", ctypes.c_int32),
        ("saleh_valence", ctypes.c_int32 * 3),
        ("B2", ctypes.c_double),
        ("B3", ctypes.c_double),
        ("delta", ctypes.c_double),
        ("regularisation_delta", ctypes.c_double),
        ("delta_AA", ctypes.c_double),
        ("delta_BB", ctypes.c_double),
        ("density_conversion_factor", ctypes.c_double),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int32),
        ("N", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("mobility_type", ctypes.c_int32),
        ("dt", ctypes.c_double),
        ("dx", ctypes.c_double),
        ("k", ctypes.c_double * CHGB_MAX_SPECIES),
        ("M", ctypes.c_double),
        ("splitting_S", ctypes.c_double),
        ("use_dealias", ctypes.c_int32),
        ("kernel_variant", ctypes.c_int32),
        ("model", ModelParams),
        ("rho_min", ctypes.c_double),
        ("gel_phi_critical", ctypes.c_double),
        ("gel_c0", ctypes.c_double),
        ("gel_M_c", ctypes.c_double),
        ("gel_beta_delta_F", ctypes.c_double),
        ("use_gmres", ctypes.c_int32),
        ("gmres_restart", ctypes.c_int32),
        ("gmres_max_iter", ctypes.c_int32),
        ("gmres_tol", ctypes.c_double),
    ]

    @property
    def n_species(self) -> int:
        return int(self.model.n_species)

    @property
    def bins(self) -> int:
        return int(self.N) ** int(self.dims)

    def copy(self) -> "Params":
        out = Params()
        ctypes.pointer(out)[0] = self
        return out


# Every symbol include/chgb.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "chgb_abi_version": (ctypes.c_int, []),
    "chgb_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(_P)]),
    "chgb_destroy": (ctypes.c_int, [_P]),
    "chgb_upload": (ctypes.c_int, [_P, _D, _D]),
    "chgb_step": (ctypes.c_int, [_P, ctypes.c_int64]),
    "chgb_download": (ctypes.c_int, [_P, _D, _D]),
    "chgb_observables": (ctypes.c_int, [_P, _D, _D, ctypes.POINTER(ctypes.c_int32)]),
    "chgb_pressure": (ctypes.c_int, [_P, _D, _D]),
    "chgb_set_stream": (ctypes.c_int, [_P, _P]),
    "chgb_synchronize": (ctypes.c_int, [_P]),
    "chgb_device_rho": (ctypes.c_int, [_P, ctypes.POINTER(_D)]),
    "chgb_launch_count": (ctypes.c_int64, [_P]),
    "chgb_bounds_report": (ctypes.c_int, [ctypes.POINTER(ctypes.c_ulonglong)]),
    "chgb_kernel_variant": (ctypes.c_int, [_P]),
    "chgb_last_error": (ctypes.c_char_p, [_P]),
    "chgb_der_bulk_free_energy": (ctypes.c_int, [ctypes.POINTER(ModelParams), _P, _P, ctypes.c_int64, _P]),
    "chgb_set_mobility": (ctypes.c_int, [ctypes.POINTER(ModelParams), _P, ctypes.c_double, _P,
                                         ctypes.c_int64, _P]),
    "chgb_observables_noalloc": (ctypes.c_int, [ctypes.POINTER(Params), _P, _P, _P]),
    "chgb_batch_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int32, ctypes.POINTER(_P)]),
    "chgb_batch_destroy": (ctypes.c_int, [_P]),
    "chgb_batch_size": (ctypes.c_int, [_P]),
    "chgb_batch_upload": (ctypes.c_int, [_P, ctypes.c_int32, _D]),
    "chgb_batch_step": (ctypes.c_int, [_P, ctypes.c_int64]),
    "chgb_batch_synchronize": (ctypes.c_int, [_P]),
    "chgb_batch_download": (ctypes.c_int, [_P, ctypes.c_int32, _D]),
    "chgb_batch_replica": (_P, [_P, ctypes.c_int32]),
    "chgb_batch_launch_count": (ctypes.c_int64, [_P]),
    "chgb_batch_euler_tile": (ctypes.c_int, [_P]),
    "chgb_structure_factor_bins": (ctypes.c_int, [ctypes.c_int32]),
    "chgb_structure_factor": (ctypes.c_int, [_P, ctypes.c_int32, _D, ctypes.c_int32]),
    "chgb_adjoint_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int64, ctypes.c_int32,
                                           ctypes.POINTER(_P)]),
    "chgb_adjoint_destroy": (ctypes.c_int, [_P]),
    "chgb_adjoint_forward": (ctypes.c_int, [_P, _D, _D, _D]),
    "chgb_adjoint_backward": (ctypes.c_int, [_P, _D, _D, _D, _D]),
    "chgb_adjoint_launch_count": (ctypes.c_int64, [_P]),
}

_LIB = None


class ChgbError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"chgb error {code}: {message}")
        self.code = code


def load_library(path: os.PathLike | None = None) -> ctypes.CDLL:
    """Load libchgb.so (built in-tree by __graft_entry__.build()).

    Raises FileNotFoundError when the library has not been built: the CUDA
    path is the only implementation.
    """
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} not found: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.chgb_abi_version() != CHGB_ABI_VERSION:
        raise RuntimeError("libchgb ABI version mismatch")
    if path is None:
        _LIB = lib
    return lib


def check(lib: ctypes.CDLL, code: int, handle=None) -> None:
    if code != CHGB_OK:
        msg = lib.chgb_last_error(handle)
        raise ChgbError(code, msg.decode() if msg else "")


def declared_symbols(header: os.PathLike = HEADER_PATH) -> list[str]:
    """Names of the functions include/chgb.h declares (parsed from the text)."""
    import re
    text = Path(header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(chgb_[a-z0-9_]+)\s*\(", text)))
