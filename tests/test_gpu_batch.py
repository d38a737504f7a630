"""Batched mode: replicas of different N, parameters and integrators stepped
together give the same bits as each replica stepped alone, and match the CPU
oracle to 1e-12 relative max-norm."""
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np
import pytest

import oracle
from chgb import abi, config
from chgb.sim import Batch, CahnHilliard
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu


def mixed_replicas(seed=0):
    rng = np.random.default_rng(seed)
    reps = []
    for N in (16, 32, 64, 128, 64, 32):
        eps, k = rng.uniform(0.5, 1.0), rng.uniform(0.5, 1.4)
        reps.append(config.params(2, N, "euler", "landau", dt=0.01, k=k, epsilon=eps))
    for N in (8, 64, 128, 256, 32):
        eps, k = rng.uniform(0.5, 1.0), rng.uniform(0.5, 2.0)
        reps.append(config.params(2, N, "pseudospectral", "landau", dt=0.05, k=k, epsilon=eps,
                                  use_dealias=bool(N == 64)))
    reps.append(config.params(2, 32, "euler", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, B3=1e7, delta_AA=1e4,
                              delta_BB=2e4))
    reps.append(config.params(2, 16, "pseudospectral", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, delta_AA=1e4,
                              delta_BB=2e4))
    reps.append(config.params(3, 16, "euler", "landau", dt=0.005, k=1.0, epsilon=0.9))          # runs loose
    reps.append(config.params(1, 64, "pseudospectral", "landau", dt=0.05, k=1.0, epsilon=0.9))  # runs loose
    reps.append(config.params(2, 8, "euler", "landau", dt=0.01, k=1.0, epsilon=0.9))            # N < 16: loose
    for integ in ("euler_mobility", "pseudospectral_mobility"):                                 # gel: loose
        q = config.params(2, 32, integ, "landau", dt=0.01, k=1.0, epsilon=0.9, mobility="gel", use_dealias=True)
        q.gel_phi_critical, q.gel_c0, q.gel_M_c = 0.3, 0.1, 20.0
        q.gel_beta_delta_F = 10.0 / (1.0 - 0.9) - np.log(24000.0)
        reps.append(q)
    fields = []
    for i, p in enumerate(reps):
        S = p.model.n_species
        if S == 3:
            rho = config.init_density(p.dims, p.N, [9e-5, 7e-5, 3e-5], seed=100 + i)
        else:
            rho = config.init_density(p.dims, p.N, [0.0], initial_A=0.01, seed=100 + i) + rng.uniform(-0.4, 0.4)
        fields.append(rho)
    return reps, fields


def single_box(p):
    """The replica's parameters for a single box.  Explicit replicas run the
    single box's bit-identical kernel variants (1-4, here 1), as the batch's
    work-list kernels do; left to kernel_variant 0, a large Landau box would
    run block fixed point (variant 5), which agrees with them to round-off
    only."""
    q = p.copy()
    if q.integrator == abi.INTEGRATORS["euler"] and q.kernel_variant == 0:
        q.kernel_variant = 1
    return q


def alone(p, rho, steps):
    sim = CahnHilliard(single_box(p), rho)
    sim.evolve(steps)
    out = sim.sync()
    sim.close()
    return out


def test_batch_matches_single_boxes_and_oracle():
    reps, fields = mixed_replicas()
    steps = 75                                   # 2 graphs of 32 + 11 batched steps (+ the fresh first step)
    with Batch(reps) as b:
        for i, f in enumerate(fields):
            b.upload(i, f)
        b.step(steps)
        got = [b.download(i) for i in range(len(reps))]
        assert b.euler_tile in (16, 32, 64)
    for i, (p, f) in enumerate(zip(reps, fields)):
        ref_alone = alone(p, f, steps)
        assert np.array_equal(got[i], ref_alone), f"replica {i} differs from the single-box run"
        o = oracle.OracleSim(p, f)
        o.step(steps)
        assert rel_maxnorm(got[i], o.rho()) <= 1e-12, i


def test_batch_reupload_and_repeated_steps():
    reps, fields = mixed_replicas(seed=3)
    with Batch(reps) as b:
        for i, f in enumerate(fields):
            b.upload(i, f)
        b.step(33)                               # odd: leaves the euler group at parity 1
        mid = [b.download(i) for i in range(len(reps))]
        # re-upload two replicas (one euler, one pseudospectral) mid-run
        b.upload(1, fields[1])
        b.upload(7, fields[7])
        b.step(40)
        out = [b.download(i) for i in range(len(reps))]
        mass, fe, nan = b.observables(2)
        assert not nan
    for i, (p, f) in enumerate(zip(reps, fields)):
        if i in (1, 7):
            want = alone(p, f, 40)
        else:
            sim = CahnHilliard(single_box(p), f)
            sim.evolve(33)
            assert np.array_equal(sim.sync(), mid[i])
            sim.evolve(40)
            want = sim.sync()
        assert np.array_equal(out[i], want), i


def test_batch_launch_count_is_per_group():
    reps = [config.params(2, 64, "euler", "landau", dt=0.01, epsilon=0.9) for _ in range(5)]
    reps += [config.params(2, 64, "pseudospectral", "landau", dt=0.05, epsilon=0.9) for _ in range(3)]
    with Batch(reps) as b:
        for i, p in enumerate(reps):
            b.upload(i, config.init_density(2, 64, [0.0], seed=i))
        b.step(1)                                # fresh: euler batched (1) + 3 single pseudospectral steps (2 each)
        n1 = b.launches
        b.step(64)                               # 64 steps x (1 euler + 2 pseudospectral) launches
        assert b.launches - n1 == 64 * 3


def _benchmark_replicas():
    """The batch configuration exactly as bench.py times it: 256 replicas,
    N uniform in {64, 128, 256, 512}, half euler and half pseudospectral."""
    import sys
    repo = str(Path(__file__).resolve().parent.parent)
    if repo not in sys.path:
        sys.path.insert(0, repo)
    import bench
    return bench.batch_replicas()


def _oracle_rho(p, f, steps):
    o = oracle.OracleSim(p, f)
    o.step(steps)
    out = o.rho()
    o.close()
    return out


def test_benchmark_batch_configuration():
    """The 256-replica benchmark batch (21.9 M cells) for 100 steps: every
    replica equals its single-box run bit for bit, and one euler and one
    pseudospectral replica of each N match the oracle to 1e-12."""
    reps, fields = _benchmark_replicas()
    assert len(reps) == 256 and {p.N for p in reps} == {64, 128, 256, 512}
    steps = 100
    picks = {}
    for i, p in enumerate(reps):
        picks.setdefault((p.N, p.integrator), i)
    assert len(picks) == 8
    with ThreadPoolExecutor(max_workers=len(picks)) as ex:
        futs = {i: ex.submit(_oracle_rho, reps[i], fields[i], steps) for i in picks.values()}
        with Batch(reps) as b:
            for i, f in enumerate(fields):
                b.upload(i, f)
            b.step(steps)
            got = [b.download(i) for i in range(len(reps))]
        for i, (p, f) in enumerate(zip(reps, fields)):
            assert np.array_equal(got[i], alone(p, f, steps)), f"replica {i} (N={p.N}) differs from its single-box run"
        for i, fut in futs.items():
            assert rel_maxnorm(got[i], fut.result()) <= 1e-12, (i, reps[i].N, reps[i].integrator)
