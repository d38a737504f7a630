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
from chgb.sim import Batch, CahnHilliard

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
    elif name in ("ps", "ps_dealias"):
        p = config.params(dims, N, "pseudospectral", "landau", dt=0.05, k=1.0, epsilon=0.9,
                          use_dealias=name == "ps_dealias")
        rho0 = config.init_density(dims, N, [0.0], initial_A=0.3, seed=13)
    elif name == "ps_saleh":
        p = config.params(dims, N, "pseudospectral", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, delta_AA=1e4,
                          delta_BB=2e4)
        rho0 = config.init_density(dims, N, [9e-5, 7e-5, 3e-5], seed=13)
    elif name in ("psmob", "gmres"):   # pseudospectral_mobility, gel mobility (M0 splitting or GMRES)
        p = config.params(dims, N, "pseudospectral_mobility", "landau", dt=0.01, k=1.0, epsilon=0.9, mobility="gel",
                          S=0.3, use_dealias=True)
        p.gel_phi_critical, p.gel_c0, p.gel_M_c = 0.3, 0.1, 20.0
        p.gel_beta_delta_F = 10.0 / (1.0 - 0.9) - np.log(24000.0)
        if name == "gmres":
            p.use_gmres, p.gmres_restart, p.gmres_max_iter, p.gmres_tol = 1, 8, 40, 1e-11
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
    # the transforms (spectral.cu): rows, columns, both 3D column axes, three species, the
    # variable-mobility passes
    ("ps", 1, 64, 1, 5), ("ps", 2, 8, 1, 5), ("ps", 2, 64, 1, 5), ("ps", 2, 1024, 1, 3), ("ps", 2, 4096, 1, 2),
    ("ps_dealias", 2, 128, 1, 3), ("ps", 3, 16, 1, 3), ("ps", 3, 128, 1, 2), ("ps_saleh", 2, 32, 1, 3),
    ("ps_saleh", 3, 16, 1, 2), ("psmob", 2, 64, 1, 3), ("psmob", 3, 16, 1, 2), ("gmres", 2, 32, 1, 2),
])
def test_kernels_stay_in_bounds(bc_lib, name, dims, N, variant, steps):
    """One case through the bounds-check build, then through the normal one."""
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


def test_batch_stays_in_bounds(bc_lib):
    """The batch's work-list kernels (euler tiles, row and column passes of
    many replicas) through the bounds-check build: clean, and the normal
    build's bits."""
    reps, fields = [], []
    for i, N in enumerate((16, 32, 64, 128, 256)):
        reps.append(config.params(2, N, "euler", "landau", dt=0.01, k=1.0, epsilon=0.9))
        reps.append(config.params(2, N, "pseudospectral", "landau", dt=0.05, k=1.0, epsilon=0.9))
        for _ in range(2):
            fields.append(config.init_density(2, N, [0.0], initial_A=0.3, seed=40 + i))
    out = {}
    _report(bc_lib)
    for key, lib in (("bc", bc_lib), ("plain", None)):
        with Batch(reps, lib=lib) as b:
            for i, f in enumerate(fields):
                b.upload(i, f)
            b.step(7)
            out[key] = [b.download(i) for i in range(len(reps))]
    assert _report(bc_lib) == 0
    for a, c in zip(out["bc"], out["plain"]):
        assert np.array_equal(a, c)
