"""chgb_observables_noalloc: the observables entry point for callers that
cannot allocate device memory when they need the mass and free energy (their
pool already owns HBM, or their loop cannot pay for cudaMalloc/cudaFree).

It is checked through the C ABI against the existing entry point
chgb_observables on two calls in a row (the second call reuses the library's
fixed scratch array), within the tolerances of the other observables tests.
This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from chgb import abi, config
from chgb.sim import CahnHilliard

pytestmark = pytest.mark.gpu


def _noalloc(lib, p, d_rho_ptr):
    import torch
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    code = lib.chgb_observables_noalloc(ctypes.byref(p), ctypes.c_void_p(d_rho_ptr), ctypes.c_void_p(out.data_ptr()),
                                        None)
    abi.check(lib, code)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _field(case):
    if case == "landau2d":
        p = config.params(2, 128, "euler", "landau", dt=0.01, k=1.0, epsilon=0.9)
        rho0 = config.init_density(2, 128, [-0.2], initial_A=0.3, seed=31)
        steps = 30
    else:
        p = config.params(3, 16, "euler", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, B3=1e7, delta_AA=1e4,
                          delta_BB=2e4, saleh_valence=(4, 4, 2))
        rho0 = config.init_density(3, 16, [9e-5, 7e-5, 3e-5], seed=5)
        steps = 10
    sim = CahnHilliard(p, rho0)
    sim.evolve(steps)
    return p, sim, rho0


def test_noalloc_matches_chgb_observables_two_calls():
    lib = abi.load_library()
    results = []
    for case in ("landau2d", "saleh3d"):           # two calls in a row, different fields
        p, sim, rho0 = _field(case)
        mass, fe, nan = sim.observables()           # the existing entry point
        sim.synchronize()
        got = _noalloc(lib, p, sim.device_rho())
        results.append((got, mass, fe))
        assert not nan
        assert abs(got[0] - mass) <= 1e-13 * np.abs(rho0).mean() * p.dx ** 3 + 1e-300
        assert abs(got[1] - fe) <= 1e-12 * abs(fe)
        sim.close()
    # the first field again: the scratch keeps the last call's contents, which must not leak in
    p, sim, rho0 = _field("landau2d")
    sim.synchronize()
    again = _noalloc(lib, p, sim.device_rho())
    assert np.array_equal(again, results[0][0])


def test_noalloc_rejects_fields_above_the_scratch_limit():
    lib = abi.load_library()
    p = config.params(3, 512, "euler", "landau", dt=0.01, epsilon=0.9)   # 134 M cells > 16.7 M
    dummy = ctypes.c_void_p(256)        # rejected before any device access
    code = lib.chgb_observables_noalloc(ctypes.byref(p), dummy, dummy, None)
    assert code == abi.CHGB_ERR_INVALID
    assert "exceeds the no-allocation scratch" in lib.chgb_last_error(None).decode()
