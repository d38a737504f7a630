"""GPU parity of `pseudospectral_mobility` (PseudospectralMobilityCPU's
simple path: the constant reference mobility M0 = max M semi-implicit, the
remainder explicit through real-space fluxes) against the reference's own
runs and the CPU oracle, 1e-12 relative max-norm."""
import numpy as np
import pytest

import oracle
from chgb import abi, config
from chgb.sim import CahnHilliard
from conftest import rel_maxnorm, setup_case

pytestmark = pytest.mark.gpu
TOL = 1e-12


def gel(p):
    p.mobility_type = abi.MOBILITIES["gel"]
    p.gel_phi_critical, p.gel_c0, p.gel_M_c = 0.3, 0.1, 20.0
    p.gel_beta_delta_F = 10.0 / (1.0 - 0.9) - np.log(24000.0)
    return p


def run_both(p, rho0, steps):
    sim = CahnHilliard(p, rho0)
    sim.evolve(steps)
    got, mob = sim.sync(with_mobility=True)
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    return sim, ref, got, mob


def test_reference_dumps_pseudospectral_mobility(ref_dumps):
    n = 0
    for case in ref_dumps:
        st, p, rho0 = setup_case(case)
        if p.integrator != abi.INTEGRATORS["pseudospectral_mobility"]:
            continue
        sim = CahnHilliard(p, rho0)
        sim.evolve(case["steps"])
        got, mob = sim.sync(with_mobility=True)
        assert rel_maxnorm(got, case["final"]) <= TOL, case["name"]
        if case["mobility"] is not None:
            assert rel_maxnorm(mob, case["mobility"]) <= TOL, case["name"]
        n += 1
    assert n >= 7


@pytest.mark.parametrize("dims,N,dealias,S,steps", [(2, 64, True, 0.0, 200), (2, 128, False, 0.4, 100),
                                                    (3, 32, True, 0.0, 40), (1, 256, True, 0.2, 200)])
def test_gel_matches_oracle(dims, N, dealias, S, steps):
    p = gel(config.params(dims, N, "pseudospectral_mobility", "landau", dt=0.02, k=1.0, epsilon=0.9, S=S,
                          use_dealias=dealias))
    rho0 = config.init_density(dims, N, [-0.1], initial_A=0.3, seed=3 + N)
    sim, ref, got, mob = run_both(p, rho0, steps)
    assert rel_maxnorm(got, ref.rho()) <= TOL
    assert rel_maxnorm(mob, ref.mobility()) <= TOL
    # mass is carried by the k = 0 mode, which the update leaves untouched
    assert abs(got.mean() - rho0.mean()) <= 1e-13 * max(1.0, np.abs(rho0).max())


def test_saleh_constant_mobility_matches_oracle():
    """Three species, constant mobility: the flux stages vanish exactly."""
    p = config.params(2, 32, "pseudospectral_mobility", "saleh", dt=1e-6, dx=10.0, k=[1e6, 2e6, 5e5], M=1.0,
                      B2=2190.0, B3=1e7, delta_AA=1e4, delta_BB=2e4)
    rho0 = config.init_density(2, 32, [9e-5, 7e-5, 3e-5], seed=5)
    sim, ref, got, _ = run_both(p, rho0, 30)
    assert rel_maxnorm(got, ref.rho()) <= TOL


@pytest.mark.parametrize("dims,N", [(2, 16), (2, 8), (3, 8)])
def test_saleh_regularised_mobility_matches_oracle(dims, N):
    """Three species with a field mobility each (regularised, M rho / (rho +
    rho_min)): the flux stage subtracts each species' own M0 inside the row
    pass.  Small boxes: one to four threads per transform line."""
    p = config.params(dims, N, "pseudospectral_mobility", "saleh", dt=1e-6, dx=10.0, k=[1e6, 2e6, 5e5], M=1.0,
                      B2=2190.0, B3=1e7, delta_AA=1e4, delta_BB=2e4)
    p.mobility_type = abi.MOBILITIES["regularised"]
    p.M, p.rho_min = 0.5, 2e-5
    rho0 = config.init_density(dims, N, [9e-5, 7e-5, 3e-5], seed=6 + N)
    sim, ref, got, mob = run_both(p, rho0, 30)
    assert rel_maxnorm(got, ref.rho()) <= TOL
    assert rel_maxnorm(mob, ref.mobility()) <= TOL
    assert not np.array_equal(got, rho0)


def test_wertheim_free_energy_mobility_matches_oracle():
    p = config.params(3, 16, "pseudospectral_mobility", "simple_wertheim", dt=1e-4, dx=10.0, k=1e6, M=1.0,
                      mobility="free_energy", valence=4, B2=2190.0, delta=config.delta_value(
                          {"T": 300, "deltaH": -42200, "deltaS": -119.1, "salt": 0.5, "sticky_size": 6}, "d"))
    rho0 = config.init_density(3, 16, [1.107e-5], seed=9)
    sim, ref, got, mob = run_both(p, rho0, 30)
    assert rel_maxnorm(got, ref.rho()) <= TOL
    assert rel_maxnorm(mob, ref.mobility()) <= TOL


def test_graph_decompositions_agree():
    p = gel(config.params(2, 64, "pseudospectral_mobility", "landau", dt=0.02, k=1.0, epsilon=0.9))
    rho0 = config.init_density(2, 64, [0.0], initial_A=0.2, seed=1)
    a = CahnHilliard(p, rho0)
    a.evolve(100)
    b = CahnHilliard(p, rho0)
    for n in (1, 37, 62):
        b.evolve(n)
    assert np.array_equal(a.sync(), b.sync())


@pytest.mark.parametrize("dims,N,dealias,steps", [(2, 64, True, 20), (3, 16, False, 8)])
def test_gmres_path_matches_oracle(dims, N, dealias, steps):
    """pseudospectral.use_gmres = true: restarted, left-preconditioned GMRES
    per step.  The inner products are summed in another order than the
    oracle's sequential loops, so the iterates agree to round-off."""
    p = gel(config.params(dims, N, "pseudospectral_mobility", "landau", dt=0.02, k=1.0, epsilon=0.9, S=0.3,
                          use_dealias=dealias))
    p.use_gmres, p.gmres_restart, p.gmres_max_iter, p.gmres_tol = 1, 10, 200, 1e-11
    rho0 = config.init_density(dims, N, [0.05], initial_A=0.3, seed=17)
    sim, ref, got, mob = run_both(p, rho0, steps)
    err = rel_maxnorm(got, ref.rho())
    print(f"GMRES path, {dims}D N={N}: relative max-norm {err:.2e}")
    assert err <= TOL
    assert rel_maxnorm(mob, ref.mobility()) <= TOL


@pytest.mark.parametrize("restart,max_iter,tol", [(2, 200, 1e-11), (3, 7, 1e-11), (10, 25, 0.0), (30, 200, 1e-10)])
def test_gmres_stopping_rules_match_oracle(restart, max_iter, tol):
    """The device-side restart and Arnoldi loops follow the reference's
    stopping rules: restart length 2 (many restart cycles), an iteration limit
    reached before the tolerance (7, and 25 with tol = 0), the default restart
    length 30.  The oracle runs the reference's loop."""
    p = gel(config.params(2, 32, "pseudospectral_mobility", "landau", dt=0.02, k=1.0, epsilon=0.9, S=0.2,
                          use_dealias=True))
    p.use_gmres, p.gmres_restart, p.gmres_max_iter, p.gmres_tol = 1, restart, max_iter, tol
    rho0 = config.init_density(2, 32, [0.0], initial_A=0.3, seed=23)
    sim, ref, got, _ = run_both(p, rho0, 6)
    assert rel_maxnorm(got, ref.rho()) <= TOL, (restart, max_iter, tol)


def test_gmres_benchmark_case_and_launch_count():
    """The benchmarked GMRES configuration (2D N=256, restart 10, tol 1e-11):
    parity with the oracle, and the launch count includes the kernels of the
    device-side loops (more than the fixed per-step part)."""
    p = gel(config.params(2, 256, "pseudospectral_mobility", "landau", dt=0.02, k=1.0, epsilon=0.9, S=0.3))
    p.use_gmres, p.gmres_restart, p.gmres_max_iter, p.gmres_tol = 1, 10, 200, 1e-11
    rho0 = config.init_density(2, 256, [-0.1], initial_A=0.3, seed=41)
    sim = CahnHilliard(p, rho0)
    sim.evolve(1)
    sim.synchronize()
    one = sim.launches
    sim.evolve(4)
    got = sim.sync()
    five = sim.launches
    ref = oracle.OracleSim(p, rho0)
    ref.step(5)
    assert rel_maxnorm(got, ref.rho()) <= TOL
    assert five > one > 100          # each step runs tens of kernels per Arnoldi step
    sim.close()
