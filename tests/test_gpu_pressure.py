"""Pressure (chgb_pressure): the Landau pressure field and average pressure of
the reference's CahnHilliard::pressure() / average_pressure().

* Against the reference's own values on every Landau case of the full-precision
  dumps (euler, pseudospectral, gel mobility; 1D/2D/3D), before and after the
  run, at 1e-12.
* Against the oracle on a full-size 2D N=1024 pseudospectral quench and the 3D
  N=256 euler field after 100 steps, at 1e-12.
* Other models return CHGB_ERR_UNSUPPORTED, the reference's critical().
"""
import numpy as np
import pytest

import oracle
from chgb import abi, config
from chgb.sim import CahnHilliard
from conftest import rel_maxnorm, setup_case

pytestmark = pytest.mark.gpu
TOL = 1e-12


def test_pressure_matches_reference_dumps(ref_dumps):
    n = 0
    for case in ref_dumps:
        if case["pressure"] is None:
            continue
        st, p, rho0 = setup_case(case)
        sim = CahnHilliard(p, rho0)
        before = sim.average_pressure()
        assert abs(before - case["avg_pressure"][0]) <= TOL * abs(case["avg_pressure"][0]), case["name"]
        sim.evolve(case["steps"])
        field = sim.pressure()
        avg = sim.average_pressure()
        sim.close()
        assert rel_maxnorm(field, case["pressure"]) <= TOL, case["name"]
        assert abs(avg - case["avg_pressure"][1]) <= TOL * abs(case["avg_pressure"][1]), (case["name"], avg)
        # the field and the average come from one pass: the mean of the field is the average
        assert abs(field.sum() / p.bins - avg) <= 1e-12 * np.abs(field).max()
        n += 1
    assert n >= 10


@pytest.mark.parametrize("dims,N,integrator,dt,rho_mean", [
    (2, 1024, "pseudospectral", 0.05, -0.3),
    (3, 256, "euler", 0.005, 0.0),
])
def test_pressure_full_size_matches_oracle(dims, N, integrator, dt, rho_mean):
    p = config.params(dims, N, integrator, "landau", dt=dt, k=1.0, M=1.0, epsilon=0.9)
    rho0 = config.init_density(dims, N, [rho_mean], initial_A=0.05, seed=31)
    sim = CahnHilliard(p, rho0)
    sim.evolve(20)
    got_field, got_avg = sim.pressure(), sim.average_pressure()
    state = sim.sync()
    sim.close()
    ref = oracle.OracleSim(p, state)        # the oracle's pressure of the GPU's own state
    assert rel_maxnorm(got_field, ref.pressure()) <= TOL
    want = ref.average_pressure()
    assert abs(got_avg - want) <= TOL * abs(want)
    ref.close()


@pytest.mark.parametrize("model", ["simple_wertheim", "saleh"])
def test_pressure_is_unsupported_for_other_models(model):
    if model == "saleh":
        p = config.params(2, 16, "euler", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, delta_AA=1e4, delta_BB=2e4)
        rho0 = config.init_density(2, 16, [9e-5, 7e-5, 3e-5], seed=1)
    else:
        p = config.params(2, 16, "euler", "simple_wertheim", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, delta=1e4,
                          valence=4)
        rho0 = config.init_density(2, 16, [5e-5], seed=1)
    sim = CahnHilliard(p, rho0)
    v = np.zeros(1)
    code = sim.lib.chgb_pressure(sim._h, None, v.ctypes.data_as(abi._D))
    assert code == abi.CHGB_ERR_UNSUPPORTED
    assert "pressure coupling" in sim.lib.chgb_last_error(sim._h).decode()
    sim.close()
