"""GPU parity tests of the `pseudospectral` integrator (own FP64 FFT) against
the CPU oracle (FFTW semantics, src/integrators/PseudospectralCPU.cpp) and the
reference's own full-precision dumps.  Tolerance 1e-12 relative max-norm."""
import numpy as np
import pytest

import oracle
from chgb import abi, config
from chgb.sim import CahnHilliard
from conftest import rel_maxnorm, setup_case

pytestmark = pytest.mark.gpu
TOL = 1e-12


def run_both(p, rho0, steps):
    sim = CahnHilliard(p, rho0)
    sim.evolve(steps)
    got = sim.sync()
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    return sim, ref, got, ref.rho()


@pytest.mark.parametrize("dims,N,dt,k,M,S,dealias,rho_mean,steps", [
    (1, 64, 0.05, 1.0, 1.0, 0.0, False, 0.0, 100),
    (1, 4, 0.05, 1.0, 1.0, 0.0, False, 0.0, 20),
    (1, 2048, 0.05, 0.5, 1.0, 0.3, True, -0.3, 50),
    (2, 64, 0.05, 1.0, 1.0, 0.0, False, 0.0, 100),
    (2, 64, 0.05, 1.0, 1.0, 0.5, True, -0.3, 100),
    (2, 4, 0.05, 1.0, 1.0, 0.0, False, 0.0, 20),
    (2, 8, 0.05, 1.0, 1.0, 0.0, True, 0.0, 20),
    (2, 128, 0.05, 1.3, 0.8, 0.0, False, 0.1, 50),
    (2, 512, 0.05, 1.0, 1.0, 0.0, False, 0.0, 10),
    (2, 1024, 0.05, 1.0, 1.0, 0.0, False, 0.0, 5),
    (3, 16, 0.05, 1.0, 1.0, 0.0, True, 0.0, 50),
    (3, 8, 0.05, 1.0, 1.0, 0.2, False, 0.0, 20),
    (3, 32, 0.05, 0.8, 1.2, 0.0, False, -0.2, 20),
    (3, 64, 0.05, 1.0, 1.0, 0.0, False, 0.0, 5),
])
def test_landau_matches_oracle(dims, N, dt, k, M, S, dealias, rho_mean, steps):
    p = config.params(dims, N, "pseudospectral", "landau", dt=dt, k=k, M=M, S=S, use_dealias=dealias, epsilon=0.9)
    rho0 = config.init_density(dims, N, [rho_mean], seed=4242 + N)
    sim, ref, got, want = run_both(p, rho0, steps)
    assert rel_maxnorm(got, want) <= TOL
    assert abs(got.mean() - rho0.mean()) <= 1e-13 * max(1.0, np.abs(rho0).max())


def test_upload_download_roundtrip_is_exact():
    p = config.params(2, 64, "pseudospectral", "landau", dt=0.05, epsilon=0.9)
    rho0 = config.init_density(2, 64, [0.1], seed=1)
    sim = CahnHilliard(p, rho0)
    assert np.array_equal(sim.sync(), rho0)


def test_sync_between_steps_does_not_perturb():
    p = config.params(2, 64, "pseudospectral", "landau", dt=0.05, epsilon=0.9)
    rho0 = config.init_density(2, 64, [0.0], seed=2)
    a = CahnHilliard(p, rho0)
    for _ in range(5):
        a.evolve(10)
        a.sync()
        a.observables()
    b = CahnHilliard(p, rho0)
    b.evolve(50)
    assert np.array_equal(a.sync(), b.sync())


@pytest.mark.parametrize("dims,N", [(1, 32), (2, 16), (3, 8)])
def test_saleh_and_wertheim_match_oracle(dims, N):
    p = config.params(dims, N, "pseudospectral", "saleh", dt=1e-6, dx=10.0, k=[1e6, 2e6, 5e5], M=1.0, B2=2190.0,
                      B3=1e7, delta_AA=4.5e4, delta_BB=6.1e4, saleh_valence=(4, 3, 4))
    rho0 = config.init_density(dims, N, [9e-5, 7e-5, 3e-5], seed=5)
    sim, ref, got, want = run_both(p, rho0, 30)
    assert rel_maxnorm(got, want) <= TOL
    p = config.params(dims, N, "pseudospectral", "simple_wertheim", dt=1e-4, dx=10.0, k=1e6, M=0.05, valence=4,
                      B2=2190.0, delta=4.5e4)
    rho0 = config.init_density(dims, N, [1.1e-5], seed=6)
    sim, ref, got, want = run_both(p, rho0, 30)
    assert rel_maxnorm(got, want) <= TOL


def test_reference_dumps_pseudospectral(ref_dumps):
    n = 0
    for case in ref_dumps:
        st, p, rho0 = setup_case(case)
        if p.integrator != abi.INTEGRATORS["pseudospectral"]:
            continue
        sim = CahnHilliard(p, rho0)
        sim.evolve(case["steps"])
        assert rel_maxnorm(sim.sync(), case["final"]) <= TOL, case["name"]
        n += 1
    assert n >= 5


def test_observables_after_steps():
    p = config.params(2, 128, "pseudospectral", "landau", dt=0.05, k=1.0, epsilon=0.9)
    rho0 = config.init_density(2, 128, [-0.3], initial_A=0.0333333, seed=11)
    sim, ref, got, want = run_both(p, rho0, 40)
    mass, fe, nan = sim.observables()
    assert not nan
    assert abs(mass - ref.average_mass()[0]) <= 1e-13
    fe_ref = ref.average_free_energy()[0]
    assert abs(fe - fe_ref) <= 1e-12 * abs(fe_ref)


def test_nan_propagates_through_the_transforms():
    """A NaN planted in a pseudospectral field reaches the observables (the
    fixed-point transforms give NaN for a line that held one), and the handle
    stays usable."""
    p = config.params(2, 64, "pseudospectral", "landau", dt=0.05, k=1.0, epsilon=0.9)
    rho0 = config.init_density(2, 64, [0.0], seed=2)
    rho0[1000] = np.nan
    sim = CahnHilliard(p, rho0)
    sim.evolve(3)
    assert np.isnan(sim.sync()).any()
    assert sim.observables(raise_on_nan=False)[2]
    sim.upload(config.init_density(2, 64, [0.0], seed=2))
    sim.evolve(3)
    assert not sim.observables()[2]


@pytest.mark.parametrize("scale,tol", [(1e-120, 1e-12), (1e-305, 1e-9)])
def test_fields_far_from_unit_scale_match_oracle(scale, tol):
    """The per-line block exponents follow the data: a field scaled by 1e-120,
    and by 1e-305 where the smallest modes and products fall into the
    subnormal range (the FP64 oracle loses precision there too, hence the
    looser bound), match the oracle."""
    N, steps = 64, 20
    p = config.params(2, N, "pseudospectral", "landau", dt=0.05, k=1.0, epsilon=0.9, use_dealias=True)
    rho0 = config.init_density(2, N, [0.0], initial_A=0.3, seed=8) * scale
    sim = CahnHilliard(p, rho0)
    sim.evolve(steps)
    got = sim.sync()
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    want = ref.rho()
    assert np.all(np.isfinite(got))
    assert rel_maxnorm(got, want) <= tol
