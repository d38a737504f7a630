"""The bounds-check build (lib/libchgb_bc.so, csrc/euler.cu compiled with
-DCHGB_BOUNDS_CHECK): the split and block-fixed-point kernels check every
global and shared-memory index of their staging, stencil reads and stores,
record the first bad one and skip its access.  Every launch shape those
kernels take -- the smallest boxes (one tile across), 3D 8- and 16-plane z
chunks, 2D tiles of 32 x 16 and 32 x 32, the three-species and field-mobility
split kernels -- runs clean, and gives the normal build's bits."""
import ctypes
import sys
from pathlib import Path

import numpy as np
import pytest

from chgb import abi, config
from chgb.sim import CahnHilliard

pytestmark = pytest.mark.gpu

PKG = Path(__file__).resolve().parent.parent / "cahn-hilliard_gb300"


@pytest.fixture(scope="module")
def bc_lib():
    sys.path.insert(0, str(PKG))
    import build
    return abi.load_library(build.build_bounds_check_library())


def _report(lib):
    first = ctypes.c_ulonglong(1)
    assert lib.chgb_bounds_report(ctypes.byref(first)) == abi.CHGB_OK
    return first.value


def _case(name, dims, N):
    if name == "landau":
        p = config.params(dims, N, "euler", "landau", dt=0.01 if dims == 2 else 0.005, k=1.0, epsilon=0.9)
        rho0 = config.init_density(dims, N, [0.0], initial_A=0.3, seed=13)
    elif name == "saleh":
        p = config.params(dims, N, "euler", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, B3=1e7, delta_AA=1e4,
                          delta_BB=2e4)
        rho0 = config.init_density(dims, N, [9e-5, 7e-5, 3e-5], seed=13)
    else:   # simple_wertheim euler_mobility with the free-energy mobility
        p = config.params(dims, N, "euler_mobility", "simple_wertheim", dt=1e-4, dx=10.0, k=1e6, M=1.0,
                          mobility="free_energy", valence=4, B2=2190.0, delta=4.5168e4)
        rho0 = config.init_density(dims, N, [1.107e-5], seed=13)
    return p, rho0


@pytest.mark.parametrize("name,dims,N,variant,steps", [
    ("landau", 2, 32, 2, 9), ("landau", 2, 32, 5, 9), ("landau", 2, 64, 2, 9), ("landau", 2, 512, 5, 5),
    ("landau", 2, 2048, 5, 3), ("landau", 3, 32, 2, 5), ("landau", 3, 32, 5, 5), ("landau", 3, 64, 5, 5),
    ("landau", 3, 256, 5, 3), ("saleh", 2, 32, 2, 5), ("saleh", 3, 32, 2, 3), ("wertheim", 3, 32, 2, 3),
])
def test_kernels_stay_in_bounds(bc_lib, name, dims, N, variant, steps):
    p, rho0 = _case(name, dims, N)
    p.kernel_variant = variant
    _report(bc_lib)                                  # clear
    a = CahnHilliard(p, rho0, lib=bc_lib)
    assert a.kernel_variant == variant
    a.evolve(steps)
    got = a.sync()
    a.close()
    assert _report(bc_lib) == 0
    b = CahnHilliard(p, rho0)                        # the normal build
    b.evolve(steps)
    assert np.array_equal(got, b.sync())
    b.close()
