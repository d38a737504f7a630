"""The benchmark configurations at their full sizes.

* 100-step runs against the CPU oracle at 1e-12 relative max-norm, with mass
  drift at 1e-13: 3D Landau euler N=256 (the headline), 2D Landau euler and
  pseudospectral N=1024 (critical and off-critical quench), 3D
  simple_wertheim euler_mobility N=128 with the free-energy mobility.
* Long runs through size-independent properties: mass conservation to
  round-off, the fused and split euler variants bit-identical (the
  block-fixed-point pair within 1e-13), and the
  radially averaged S(q) and free energy of long 2D runs within 1e-6 of the
  oracle's.
"""
import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle
from chgb import config
from chgb.sim import CahnHilliard
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu
TOL = 1e-12


def wertheim_config3(N):
    """examples/wertheim/simple.toml's model constants; rho_mean for ~50 % bonding."""
    return config.params(3, N, "euler_mobility", "simple_wertheim", dt=1e-4, dx=10.0, k=1e6, M=1.0,
                         mobility="free_energy", valence=4, B2=2190.0, delta=config.delta_value(
                             {"T": 300, "deltaH": -42200, "deltaS": -119.1, "salt": 0.5, "sticky_size": 6}, "d"))


STEPS = 100          # the step count of the parity bar for every full-size configuration
LANDAU_CASES = {
    # name: (dims, N, integrator, dt, rho_mean, initial_A)
    "euler3d_N256": (3, 256, "euler", 0.005, 0.0, 1e-2),
    "euler2d_N1024": (2, 1024, "euler", 0.01, 0.0, 1e-2),
    "pseudospectral2d_N1024_critical": (2, 1024, "pseudospectral", 0.05, 0.0, 1e-2),
    "pseudospectral2d_N1024_droplets": (2, 1024, "pseudospectral", 0.05, -0.3, 1.0 / 30.0),
}


def _landau_case(name):
    dims, N, integrator, dt, rho_mean, A = LANDAU_CASES[name]
    p = config.params(dims, N, integrator, "landau", dt=dt, k=1.0, M=1.0, epsilon=0.9)
    rho0 = config.init_density(dims, N, [rho_mean], initial_A=A, seed=4242)
    return p, rho0


def _wertheim_case():
    p = wertheim_config3(128)
    rho0 = config.init_density(3, 128, [1.107e-5], seed=4243)
    return p, rho0


def _oracle_run(p, rho0, steps, with_mobility=False):
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)                      # ctypes drops the GIL: the runs proceed side by side
    out = {"rho": ref.rho(), "mass": ref.average_mass()[0], "fe": ref.average_free_energy()[0]}
    if with_mobility:
        out["mobility"] = ref.mobility()
    ref.close()
    return out


@pytest.fixture(scope="module")
def oracle_runs():
    """The oracle's 100-step runs of every full-size configuration, started
    together on host threads when the first test of this module needs one
    (the 3D N=256 run takes one to two minutes on one core)."""
    ex = ThreadPoolExecutor(max_workers=len(LANDAU_CASES) + 1)
    futs = {name: ex.submit(_oracle_run, *_landau_case(name), STEPS) for name in LANDAU_CASES}
    futs["wertheim3d_N128"] = ex.submit(_oracle_run, *_wertheim_case(), STEPS, True)
    yield futs
    ex.shutdown(wait=True)


def _check_mass_drift(got, rho0):
    """Mass conservation to round-off: the mean density moves by at most
    1e-13 of the field's largest magnitude."""
    drift = abs(math.fsum(got.ravel()) - math.fsum(rho0.ravel())) / rho0.size
    assert drift <= 1e-13 * np.abs(rho0).max(), drift


@pytest.mark.parametrize("name", list(LANDAU_CASES))
def test_landau_configuration_matches_oracle(name, oracle_runs):
    """100 steps of each full-size Landau configuration: the field within
    1e-12 relative max-norm of the oracle's, mass and free energy alike, mass
    drift at round-off."""
    p, rho0 = _landau_case(name)
    sim = CahnHilliard(p, rho0)
    sim.evolve(STEPS)
    got = sim.sync()
    mass, fe, nan = sim.observables()
    sim.close()
    ref = oracle_runs[name].result()
    assert rel_maxnorm(got, ref["rho"]) <= TOL, name
    assert not nan
    assert abs(mass - ref["mass"]) <= 1e-13 * max(1.0, abs(ref["mass"]))
    assert abs(fe - ref["fe"]) <= 1e-12 * abs(ref["fe"])
    _check_mass_drift(got, rho0)


@pytest.mark.parametrize("name", ["euler3d_N256", "euler2d_N1024"])
def test_block_fixed_point_configuration_matches_oracle(name, oracle_runs):
    """The same 100 steps through kernel_variant 5 (the split pair in block
    fixed point), whichever variant the timing at create would pick."""
    p, rho0 = _landau_case(name)
    p.kernel_variant = 5
    sim = CahnHilliard(p, rho0)
    assert sim.kernel_variant == 5
    sim.evolve(STEPS)
    got = sim.sync()
    mass, fe, nan = sim.observables()
    sim.close()
    ref = oracle_runs[name].result()
    assert rel_maxnorm(got, ref["rho"]) <= TOL, name
    assert not nan
    assert abs(mass - ref["mass"]) <= 1e-13 * max(1.0, abs(ref["mass"]))
    assert abs(fe - ref["fe"]) <= 1e-12 * abs(ref["fe"])
    _check_mass_drift(got, rho0)


def test_wertheim_configuration_matches_oracle(oracle_runs):
    """3D simple_wertheim euler_mobility N=128 with the free-energy mobility,
    100 steps: density and mobility within 1e-12 of the oracle's."""
    p, rho0 = _wertheim_case()
    sim = CahnHilliard(p, rho0)
    sim.evolve(STEPS)
    got, mob = sim.sync(with_mobility=True)
    mass, fe, nan = sim.observables()
    sim.close()
    ref = oracle_runs["wertheim3d_N128"].result()
    assert rel_maxnorm(got, ref["rho"]) <= TOL
    assert rel_maxnorm(mob, ref["mobility"]) <= TOL
    assert not nan
    assert abs(mass - ref["mass"]) <= 1e-13 * abs(ref["mass"])
    assert abs(fe - ref["fe"]) <= 1e-12 * abs(ref["fe"])
    _check_mass_drift(got, rho0)


def test_headline_long_run_properties():
    """3D N=256, 1000 steps: mass conserved to round-off; the fused and the
    split variant agree to the bit, the block-fixed-point pair to 1e-13."""
    N, steps = 256, 1000
    p = config.params(3, N, "euler", "landau", dt=0.005, k=1.0, M=1.0, epsilon=0.9)
    rho0 = config.init_density(3, N, [0.0], initial_A=1e-2, seed=99)
    out = {}
    for v in (1, 2, 5):
        q = p.copy()
        q.kernel_variant = v
        sim = CahnHilliard(q, rho0)
        sim.evolve(steps)
        out[v] = sim.sync()
        sim.close()
    assert np.array_equal(out[1], out[2])
    assert rel_maxnorm(out[5], out[2]) <= 1e-13
    for v in (2, 5):
        drift = abs(out[v].mean() - rho0.mean())
        assert drift <= 1e-13 * np.abs(rho0).max()


@pytest.mark.parametrize("integrator,dt,steps,N,variant", [("pseudospectral", 0.05, 2000, 256, 0),
                                                           ("euler", 0.01, 4000, 256, 0),
                                                           ("euler", 0.01, 3000, 512, 5)])
def test_long_run_sq_and_free_energy_match_oracle(integrator, dt, steps, N, variant):
    """2D through coarsening: S(q) and the free energy within 1e-6 of the
    oracle's; N=512 runs block fixed point (kernel_variant 5) over the
    domains' growth from noise to |psi| ~ 1."""
    p = config.params(2, N, integrator, "landau", dt=dt, k=1.0, M=1.0, epsilon=0.9)
    p.kernel_variant = variant
    rho0 = config.init_density(2, N, [0.0], initial_A=1e-2, seed=777)
    sim = CahnHilliard(p, rho0)
    sim.evolve(steps)
    _, sq = sim.structure_factor()
    _, fe, _ = sim.observables()
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    _, sq_ref = oracle.radial_average_sq(ref.rho().reshape(N, N), p.dx)
    fe_ref, _ = ref.average_free_energy()
    assert np.max(np.abs(sq - sq_ref)) <= 1e-6 * np.max(sq_ref)
    assert abs(fe - fe_ref) <= 1e-6 * abs(fe_ref)
    # and the state itself stays close: coarsening does not amplify round-off much
    assert rel_maxnorm(sim.sync(), ref.rho()) <= 1e-6


# ---------------------------------------------------------------- maximum sizes

@pytest.mark.parametrize("dims,N,steps", [(3, 512, 12), (2, 16384, 4)])
def test_largest_box_properties(dims, N, steps):
    """3D N=512 and 2D N=16384 (1 and 2 GiB per field): the fused and split
    variants agree to the bit, and the mass stays put to round-off."""
    p = config.params(dims, N, "euler", "landau", dt=0.005, k=1.0, M=1.0, epsilon=0.9)
    rho0 = config.init_density(dims, N, [0.0], initial_A=1e-2, seed=5)
    out = {}
    for v in (1, 2, 5):
        q = p.copy()
        q.kernel_variant = v
        sim = CahnHilliard(q, rho0)
        sim.evolve(steps)
        out[v] = sim.sync()
        sim.close()
    assert np.array_equal(out[1], out[2])
    assert rel_maxnorm(out[5], out[2]) <= 1e-14
    for v in (2, 5):
        assert abs(out[v].mean() - rho0.mean()) <= 1e-13 * np.abs(rho0).max()


def test_largest_1d_box_matches_oracle():
    N, steps = 1 << 24, 20   # the largest 1D box
    p = config.params(1, N, "euler", "landau", dt=0.01, k=1.0, M=1.0, epsilon=0.9)
    rho0 = config.init_density(1, N, [0.0], initial_A=1e-2, seed=6)
    sim = CahnHilliard(p, rho0)
    sim.evolve(steps)
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    assert rel_maxnorm(sim.sync(), ref.rho()) <= TOL


def test_largest_pseudospectral_box_matches_oracle():
    """2D N=4096, the largest pseudospectral box (one row and one column of
    the transform fit a CTA's shared memory)."""
    N, steps = 4096, 3
    p = config.params(2, N, "pseudospectral", "landau", dt=0.05, k=1.0, M=1.0, epsilon=0.9)
    rho0 = config.init_density(2, N, [0.0], initial_A=1e-2, seed=7)
    sim = CahnHilliard(p, rho0)
    sim.evolve(steps)
    got = sim.sync()
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    assert rel_maxnorm(got, ref.rho()) <= TOL
    assert abs(got.mean() - rho0.mean()) <= 1e-13 * np.abs(rho0).max()
