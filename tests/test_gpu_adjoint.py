"""Device S(q) and the hand-written adjoint.

* S(q) against the reference's radial average (utils/sq_from_traj.py,
  restated in the oracle), 1e-12 relative.
* Adjoint gradients of L = sum_q (S(q) - S*(q))^2 against central finite
  differences (h = 1e-6, relative) of the CPU oracle's trajectory, for
  epsilon, k, M and a random direction of the initial field: <= 1e-6 relative.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle
from chgb import config
from chgb.sim import Adjoint, CahnHilliard
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("integrator,N", [("euler", 64), ("pseudospectral", 64), ("euler", 128),
                                          ("pseudospectral", 32)])
def test_structure_factor_matches_reference_definition(integrator, N):
    dt = 0.001 if integrator == "euler" else 0.05     # dx = 0.7: the explicit step needs dt < ~0.0037
    p = config.params(2, N, integrator, "landau", dt=dt, dx=0.7, k=1.0, epsilon=0.9)
    rho0 = config.init_density(2, N, [-0.2], initial_A=0.3, seed=21)
    sim = CahnHilliard(p, rho0)
    sim.evolve(40)
    q, sq = sim.structure_factor()
    qr, sr = oracle.radial_average_sq(sim.sync().reshape(N, N), p.dx)
    assert len(sq) == len(sr)
    assert np.allclose(q, qr, rtol=1e-14)
    assert np.max(np.abs(sq - sr)) <= 1e-12 * np.max(sr)


def _setup(integrator, N, steps, seed=5):
    dt = 0.01 if integrator == "euler" else 0.05
    p_true = config.params(2, N, integrator, "landau", dt=dt, k=1.3, M=1.0, epsilon=0.8)
    p = config.params(2, N, integrator, "landau", dt=dt, k=1.0, M=0.9, epsilon=0.9)
    rho0 = config.init_density(2, N, [0.0], initial_A=0.02, seed=seed)
    sim = oracle.OracleSim(p_true, rho0)
    sim.step(steps)
    _, target = oracle.radial_average_sq(sim.rho().reshape(N, N), p.dx)
    return p, rho0, target


def _fd_checks(p, rho0, steps, target, grad0, g3, h=1e-6, threads=8):
    """Central differences of the oracle loss in eps, k, M and along a field direction."""
    rng = np.random.default_rng(3)
    v = rng.standard_normal(rho0.size)
    hv = h * np.max(np.abs(rho0))
    jobs = []
    for name in ("epsilon", "k", "M"):
        for sgn in (+1, -1):
            q = p.copy()
            if name == "epsilon":
                q.model.epsilon = p.model.epsilon * (1 + sgn * h)
            elif name == "k":
                q.k[0] = p.k[0] * (1 + sgn * h)
            else:
                q.M = p.M * (1 + sgn * h)
            jobs.append((q, rho0))
    jobs.append((p, rho0 + hv * v))
    jobs.append((p, rho0 - hv * v))
    with ThreadPoolExecutor(max_workers=threads) as ex:
        vals = list(ex.map(lambda j: oracle.sq_loss_of_run(j[0], j[1], steps, target), jobs))
    fd = []
    for i, base in enumerate((p.model.epsilon, p.k[0], p.M)):
        fd.append((vals[2 * i] - vals[2 * i + 1]) / (2 * h * base))
    fd_dir = (vals[6] - vals[7]) / (2 * hv)
    adj_dir = float(np.dot(grad0, v))
    for a, f in zip(g3, fd):
        assert abs(a - f) <= 1e-6 * abs(f), (g3, fd)
    assert abs(adj_dir - fd_dir) <= 1e-6 * abs(fd_dir), (adj_dir, fd_dir)


@pytest.mark.parametrize("integrator,N,steps,K", [("euler", 32, 60, 8), ("pseudospectral", 32, 60, 7),
                                                  ("euler", 64, 45, 45), ("pseudospectral", 16, 33, 5)])
def test_adjoint_matches_finite_differences(integrator, N, steps, K):
    p, rho0, target = _setup(integrator, N, steps)
    with Adjoint(p, steps, K) as adj:
        sq, rho_t = adj.forward(rho0)
        o = oracle.OracleSim(p, rho0)
        o.step(steps)
        assert rel_maxnorm(rho_t, o.rho()) <= 1e-12
        dl_dsq = 2.0 * (sq - target)
        g0, g3 = adj.backward(dl_dsq=dl_dsq)
        # reproducible to the bit
        g0b, g3b = adj.backward(dl_dsq=dl_dsq)
        assert np.array_equal(g0, g0b) and np.array_equal(g3, g3b)
    _fd_checks(p, rho0, steps, target, g0, g3)


@pytest.mark.parametrize("N,steps,K", [(64, 45, 8), (32, 23, 23), (256, 12, 5)])
def test_two_steps_per_launch_match_one(N, steps, K):
    """euler kernel_variant 3 (two steps per launch in the forward,
    recomputation and adjoint passes) against 1 (one step per launch): the
    trajectory, S(q) and dL/drho0 are the same bits; the parameter gradients,
    summed in another order, agree to rounding.  Odd segments end with one
    single step."""
    p, rho0, target = _setup("euler", N, steps)
    out = {}
    for v in (1, 3):
        q = p.copy()
        q.kernel_variant = v
        with Adjoint(q, steps, K) as adj:
            sq, rho_t = adj.forward(rho0)
            g0, g3 = adj.backward(dl_dsq=2.0 * (sq - target))
            out[v] = (sq, rho_t, g0, g3, adj.launches)
    assert np.array_equal(out[1][0], out[3][0])
    assert np.array_equal(out[1][1], out[3][1])
    assert np.array_equal(out[1][2], out[3][2])
    assert np.allclose(out[3][3], out[1][3], rtol=1e-9, atol=0)
    segs = [min(K, steps - j) for j in range(0, steps, K)]
    saved = sum(s // 2 for s in segs)            # per pass: forward, recomputation, adjoint
    assert out[1][4] - out[3][4] == 3 * saved


@pytest.mark.parametrize("integrator", ["euler", "pseudospectral"])
def test_adjoint_field_seed_is_linear_in_the_seed(integrator):
    """dL/drho_T seeds: backward(a + b) = backward(a) + backward(b)."""
    N, steps = 32, 20
    p, rho0, target = _setup(integrator, N, steps)
    rng = np.random.default_rng(0)
    a_seed, b_seed = rng.standard_normal(N * N), rng.standard_normal(N * N)
    with Adjoint(p, steps, 6) as adj:
        adj.forward(rho0)
        ga, ea = adj.backward(dl_drho_t=a_seed)
        gb, eb = adj.backward(dl_drho_t=b_seed)
        gab, eab = adj.backward(dl_drho_t=a_seed + b_seed)
    assert np.max(np.abs(gab - (ga + gb))) <= 1e-12 * np.max(np.abs(gab))
    assert np.max(np.abs(eab - (ea + eb))) <= 1e-11 * np.max(np.abs(eab))


def test_torch_autograd_function():
    import torch
    from chgb.autograd import sq_loss, structure_factor_rollout
    N, steps = 32, 30
    p, rho0, target = _setup("euler", N, steps)
    psi0 = torch.tensor(rho0, dtype=torch.float64, requires_grad=True)
    eps = torch.tensor(p.model.epsilon, dtype=torch.float64, requires_grad=True)
    k = torch.tensor(p.k[0], dtype=torch.float64, requires_grad=True)
    M = torch.tensor(p.M, dtype=torch.float64, requires_grad=True)
    loss = sq_loss(structure_factor_rollout(psi0, eps, k, M, p, steps, 6), torch.tensor(target))
    loss.backward()
    with Adjoint(p, steps, 6) as adj:
        sq, _ = adj.forward(rho0)
        g0, g3 = adj.backward(dl_dsq=2.0 * (sq - target))
    assert np.array_equal(psi0.grad.numpy(), g0)
    assert [eps.grad.item(), k.grad.item(), M.grad.item()] == list(g3)
    assert loss.item() == pytest.approx(float(np.sum((sq - target) ** 2)), rel=1e-15)


@pytest.mark.parametrize("integrator", ["euler", "pseudospectral"])
def test_adjoint_configuration_N256_T2000(integrator):
    """The adjoint configuration: 2D Landau N=256, T=2000, a checkpoint every
    45 steps, target S* from (eps*, k*, M*) = (0.8, 1.3, 1); central
    differences (h = 1e-6) of the CPU oracle in eps, k, M and one field direction."""
    N, steps = 256, 2000
    p, rho0, target = _setup(integrator, N, steps, seed=17)
    with Adjoint(p, steps, 45) as adj:
        sq, _ = adj.forward(rho0)
        g0, g3 = adj.backward(dl_dsq=2.0 * (sq - target))
    _fd_checks(p, rho0, steps, target, g0, g3, threads=8)
