"""The bounds-check build (lib/libchgb_bc.so, csrc/euler.cu compiled with
-DCHGB_BOUNDS_CHECK): the explicit kernels check every global and
shared-memory index of their staging, stencil reads and stores (and, in the
cluster-resident box, of the neighbours' shared memory), record the first bad
one and skip its access.  Every launch shape the explicit kernels take -- the
split and block-fixed-point pairs (one-tile boxes, 3D 2- to 16-plane z chunks,
2D tiles of 32 x 16 and 32 x 32), the fused kernels' tile shapes from 4 x 4 to
32 x 32 and their 3D march, two steps per launch, the cluster-resident box,
1D, three species and the mobility fields -- runs clean, and gives the normal
build's bits."""
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
        p = config.params(dims, N, "euler", "landau", dt=0.01 if dims < 3 else 0.005, k=1.0, epsilon=0.9)
        rho0 = config.init_density(dims, N, [0.0], initial_A=0.3, seed=13)
    elif name == "saleh":
        p = config.params(dims, N, "euler", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, B3=1e7, delta_AA=1e4,
                          delta_BB=2e4)
        rho0 = config.init_density(dims, N, [9e-5, 7e-5, 3e-5], seed=13)
    elif name == "gel":   # euler_mobility with the gel mobility field (read by the step kernels)
        p = config.params(dims, N, "euler_mobility", "landau", dt=0.005, k=1.0, epsilon=0.9, mobility="gel")
        p.gel_phi_critical, p.gel_c0, p.gel_M_c = 0.3, 0.1, 20.0
        p.gel_beta_delta_F = 10.0 / (1.0 - 0.9) - np.log(24000.0)
        rho0 = config.init_density(dims, N, [-0.1], initial_A=0.2, seed=13)
    else:   # simple_wertheim euler_mobility with the free-energy mobility
        p = config.params(dims, N, "euler_mobility", "simple_wertheim", dt=1e-4, dx=10.0, k=1e6, M=1.0,
                          mobility="free_energy", valence=4, B2=2190.0, delta=4.5168e4)
        rho0 = config.init_density(dims, N, [1.107e-5], seed=13)
    return p, rho0


@pytest.mark.parametrize("name,dims,N,variant,steps", [
    # the split and block-fixed-point kernels
    ("landau", 2, 32, 2, 9), ("landau", 2, 32, 5, 9), ("landau", 2, 64, 2, 9), ("landau", 2, 512, 5, 5),
    ("landau", 2, 2048, 5, 3), ("landau", 3, 32, 2, 5), ("landau", 3, 32, 5, 5), ("landau", 3, 64, 5, 5),
    ("landau", 3, 256, 5, 3), ("saleh", 2, 32, 2, 5), ("saleh", 3, 32, 2, 3), ("wertheim", 3, 32, 2, 3),
    # the fused kernels (every tile shape), two steps per launch, the cluster-resident box, 1D
    ("landau", 2, 4, 1, 5), ("landau", 2, 8, 1, 5), ("landau", 2, 16, 1, 5), ("landau", 2, 1024, 1, 3),
    ("landau", 2, 4096, 1, 2), ("landau", 3, 8, 1, 3), ("landau", 3, 32, 1, 3), ("landau", 2, 64, 3, 6),
    ("landau", 2, 512, 3, 4), ("landau", 2, 32, 4, 7), ("landau", 2, 64, 4, 7), ("saleh", 2, 64, 4, 3),
    ("wertheim", 3, 32, 1, 3), ("gel", 2, 64, 1, 5), ("gel", 3, 32, 2, 3),
    ("landau", 1, 4, 1, 9), ("landau", 1, 64, 1, 9), ("landau", 1, 1024, 1, 9),
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
