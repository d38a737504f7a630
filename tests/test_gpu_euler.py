"""GPU parity tests of the explicit integrators (`euler`, `euler_mobility`)
against the CPU oracle and the reference's own full-precision dumps.

Tolerance: 1e-12 relative max-norm after the stated number of steps (the
parity bar for the FP64 path), mass drift <= 1e-13.
"""
import ctypes

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


LANDAU_CASES = [
    # dims, N, dt, k, M, rho_mean, steps
    (1, 64, 0.01, 1.0, 1.0, 0.0, 200),
    (1, 1024, 0.01, 0.7, 1.3, -0.2, 100),
    (1, 8, 0.01, 1.0, 1.0, 0.0, 50),
    (2, 64, 0.01, 1.0, 1.0, 0.0, 100),
    (2, 128, 0.01, 0.8, 0.7, -0.3, 100),
    (2, 16, 0.005, 1.0, 1.0, 0.1, 100),
    (2, 8, 0.005, 1.0, 1.0, 0.1, 20),
    (2, 4, 0.005, 1.0, 1.0, 0.1, 20),
    (2, 256, 0.01, 1.0, 1.0, 0.0, 20),
    (3, 32, 0.005, 1.0, 1.0, 0.0, 50),
    (3, 16, 0.005, 0.9, 1.1, -0.2, 50),
    (3, 8, 0.005, 1.0, 1.0, 0.0, 20),
    (3, 4, 0.002, 1.0, 1.0, 0.0, 20),
    (3, 64, 0.005, 1.0, 1.0, 0.0, 10),
]


@pytest.mark.parametrize("integrator", ["euler", "euler_mobility"])
@pytest.mark.parametrize("dims,N,dt,k,M,rho_mean,steps", LANDAU_CASES)
def test_landau_matches_oracle(integrator, dims, N, dt, k, M, rho_mean, steps):
    p = config.params(dims, N, integrator, "landau", dt=dt, k=k, M=M, epsilon=0.9)
    rho0 = config.init_density(dims, N, [rho_mean], seed=1000 + N + dims)
    sim, ref, got, want = run_both(p, rho0, steps)
    assert rel_maxnorm(got, want) <= TOL
    # mass drift: round-off only
    m0 = rho0.sum() / rho0.size
    assert abs(got.sum() / got.size - m0) <= 1e-13 * max(1.0, np.abs(rho0).max())


def wertheim_params(dims, N, integrator, mobility):
    # constant M = 1 would make the explicit step unstable in 3D (dt 2kM q^4 > 2); 0.05 keeps it stable
    M = 1.0 if mobility == "free_energy" else 0.05
    return config.params(dims, N, integrator, "simple_wertheim", dt=1e-4, dx=10.0, k=1e6, M=M,
                         mobility=mobility, valence=4, B2=2190.0, delta=config.delta_value(
                             {"T": 300, "deltaH": -42200, "deltaS": -119.1, "salt": 0.5, "sticky_size": 6}, "d"))


@pytest.mark.parametrize("dims,N", [(1, 64), (2, 32), (3, 16), (3, 32)])
@pytest.mark.parametrize("integrator,mobility", [("euler_mobility", "free_energy"), ("euler_mobility", "constant"),
                                                 ("euler", "constant")])
def test_simple_wertheim_matches_oracle(dims, N, integrator, mobility):
    p = wertheim_params(dims, N, integrator, mobility)
    rho0 = config.init_density(dims, N, [1.107e-5], seed=77)
    sim, ref, got, want = run_both(p, rho0, 50)
    assert rel_maxnorm(got, want) <= TOL
    _, mob = sim.sync(with_mobility=True)
    assert rel_maxnorm(mob, ref.mobility()) <= TOL


@pytest.mark.parametrize("dims,N", [(1, 32), (2, 16), (3, 8)])
@pytest.mark.parametrize("integrator", ["euler", "euler_mobility"])
def test_saleh_matches_oracle(dims, N, integrator):
    dAA = config.delta_value({"T": 293.15, "deltaH": -42200, "deltaS": -119.1, "salt": 0.5}, "a")
    dBB = config.delta_value({"T": 293.15, "deltaH": -42400, "deltaS": -120.6, "salt": 0.5}, "b")
    p = config.params(dims, N, integrator, "saleh", dt=1e-6, dx=10.0, k=[1e6, 2e6, 5e5], M=1.0, B2=2190.0,
                      B3=1e7, delta_AA=dAA, delta_BB=dBB, saleh_valence=(4, 3, 4))
    rho0 = config.init_density(dims, N, [9e-5, 7e-5, 3e-5], seed=5)
    sim, ref, got, want = run_both(p, rho0, 30)
    assert rel_maxnorm(got, want) <= TOL


def test_reference_dumps_explicit(ref_dumps):
    """Full-precision dumps of the reference's own CPU integrators."""
    n = 0
    for case in ref_dumps:
        st, p, rho0 = setup_case(case)
        if p.integrator == abi.INTEGRATORS["pseudospectral"]:
            continue
        sim = CahnHilliard(p, rho0)
        sim.evolve(case["steps"])
        got, mob = sim.sync(with_mobility=True)
        assert rel_maxnorm(got, case["final"]) <= TOL, case["name"]
        if case["mobility"] is not None:
            assert rel_maxnorm(mob, case["mobility"]) <= TOL
        n += 1
    assert n >= 8


@pytest.mark.parametrize("case", [
    (2, 64, "euler", "landau", "constant"), (3, 32, "euler", "landau", "constant"),
    (2, 128, "euler_mobility", "landau", "constant"), (3, 32, "euler_mobility", "simple_wertheim", "free_energy"),
    (2, 32, "euler", "saleh", "constant"), (3, 64, "euler", "saleh", "constant"),
    (2, 64, "euler_mobility", "landau", "gel"), (3, 32, "euler_mobility", "landau", "gel"),
    (3, 32, "euler_mobility", "simple_wertheim", "regularised"),
])
def test_fused_and_split_variants_are_bit_identical(case):
    dims, N, integrator, model, mobility = case
    if model == "landau":
        p = config.params(dims, N, integrator, model, dt=0.005, k=1.0, epsilon=0.9, mobility=mobility)
        if mobility == "gel":
            p.gel_phi_critical, p.gel_c0, p.gel_M_c = 0.3, 0.1, 20.0
            p.gel_beta_delta_F = 10.0 / (1.0 - 0.9) - np.log(24000.0)
        rho0 = config.init_density(dims, N, [-0.1], initial_A=0.2, seed=8)
    elif model == "simple_wertheim":
        p = wertheim_params(dims, N, integrator, "constant" if mobility == "regularised" else mobility)
        if mobility == "regularised":
            p.mobility_type = abi.MOBILITIES["regularised"]
            p.M, p.rho_min = 0.5, 2e-5
        rho0 = config.init_density(dims, N, [1.107e-5], seed=8)
    else:
        p = config.params(dims, N, integrator, model, dt=1e-6, dx=10.0, k=1e6, B2=2190.0, B3=1e7, delta_AA=1e4,
                          delta_BB=2e4)
        rho0 = config.init_density(dims, N, [9e-5, 7e-5, 3e-5], seed=8)
    out = {}
    two = integrator == "euler" and dims == 2 and 32 <= N <= 512   # two steps per launch
    resident = integrator == "euler" and dims == 2 and N in (32, 64)   # the box in one cluster
    for v in (1, 2) + ((3,) if two else ()) + ((4,) if resident else ()):
        q = p.copy()
        q.kernel_variant = v
        sim = CahnHilliard(q, rho0)
        assert sim.kernel_variant == v
        sim.evolve(70)                   # graphs of 64, 4 and 2 steps; variant 4: one launch
        per_step = v + (1 if mobility in ("gel", "regularised") else 0)   # + the mobility update
        assert sim.launches == {3: 35, 4: 1}.get(v, 70 * per_step)
        out[v] = sim.sync(with_mobility=True)
    for v in out:
        assert np.array_equal(out[1][0], out[v][0]) and np.array_equal(out[1][1], out[v][1]), v
    ref = oracle.OracleSim(p, rho0)
    ref.step(70)
    assert rel_maxnorm(out[2][0], ref.rho()) <= TOL


@pytest.mark.parametrize("N,model", [(64, "landau"), (32, "landau"), (64, "simple_wertheim"), (32, "saleh")])
def test_cluster_resident_box(N, model):
    """kernel_variant 4: the whole box in one 16-CTA cluster's shared memory.
    Any split of 2500 steps over chgb_step calls (a launch holds at most 1024
    steps) gives the bits of the fused kernel, and the oracle's to 1e-12."""
    if model == "landau":
        p = config.params(2, N, "euler", model, dt=0.01, k=1.0, epsilon=0.9)
        rho0 = config.init_density(2, N, [0.0], initial_A=1e-2, seed=31)
    elif model == "simple_wertheim":
        p = wertheim_params(2, N, "euler", "constant")
        rho0 = config.init_density(2, N, [1.107e-5], seed=31)
    else:
        p = config.params(2, N, "euler", model, dt=1e-6, dx=10.0, k=1e6, B2=2190.0, B3=1e7, delta_AA=1e4,
                          delta_BB=2e4)
        rho0 = config.init_density(2, N, [9e-5, 7e-5, 3e-5], seed=31)
    steps = 2500
    q = p.copy()
    q.kernel_variant = 4
    a = CahnHilliard(q, rho0)
    assert a.kernel_variant == 4
    a.evolve(steps)
    assert a.launches == 3                      # 1024 + 1024 + 452
    b = CahnHilliard(q, rho0)
    for n in (1, 2, 37, 1460, 1000):
        b.evolve(n)
    q.kernel_variant = 1
    c = CahnHilliard(q, rho0)
    c.evolve(steps)
    ra = a.sync()
    assert np.array_equal(ra, b.sync()) and np.array_equal(ra, c.sync())
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    assert rel_maxnorm(ra, ref.rho()) <= TOL


@pytest.mark.parametrize("dims,N,steps", [(2, 32, 300), (2, 256, 300), (2, 512, 120), (2, 2048, 20), (3, 32, 200),
                                          (3, 64, 100), (3, 128, 50)])
def test_block_fixed_point_variant(dims, N, steps):
    """kernel_variant 5, block fixed point (one exponent for the whole field
    per step; in 3D the split pair with mu stored as integers, in 2D one kernel
    per step): within 1e-12 of the oracle and 1e-14 of the split variant, mass
    to round-off, two kernels per step in 3D and one in 2D plus one key
    refresh per chgb_step call, and the same bits for any split of the steps
    over chgb_step calls (each call re-derives the key from the field, as the
    steps keep it)."""
    p = config.params(dims, N, "euler", "landau", dt=0.01 if dims == 2 else 0.005, k=1.0, epsilon=0.9)
    rho0 = config.init_density(dims, N, [0.0], initial_A=0.3, seed=21)
    q = p.copy()
    q.kernel_variant = 5
    a = CahnHilliard(q, rho0)
    assert a.kernel_variant == 5
    a.evolve(steps)
    assert a.launches == (2 if dims == 3 else 1) * steps + 1   # 2D: one kernel per step
    got = a.sync()
    b = CahnHilliard(q, rho0)
    left = steps
    for n in (1, steps // 3, steps // 2):
        b.evolve(n)
        left -= n
    b.evolve(left)
    assert np.array_equal(got, b.sync())
    q.kernel_variant = 2
    c = CahnHilliard(q, rho0)
    c.evolve(steps)
    assert rel_maxnorm(got, c.sync()) <= 1e-14
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    assert rel_maxnorm(got, ref.rho()) <= TOL
    assert abs(got.mean() - rho0.mean()) <= 1e-15


def test_block_fixed_point_nan_and_recovery():
    """A NaN in the field takes the FP64 sums (mode 0): it spreads as in the
    other variants, the observables report it, and after uploading a finite
    field the variant steps in block fixed point again."""
    N = 64
    p = config.params(2, N, "euler", "landau", dt=0.01, epsilon=0.9)
    p.kernel_variant = 5
    rho0 = config.init_density(2, N, [0.0], initial_A=0.5, seed=2)
    bad = rho0.copy()
    bad[77] = np.nan
    sim = CahnHilliard(p, bad)
    sim.evolve(3)
    out = sim.sync()
    assert np.isnan(out[77]) and np.isnan(out[78]) and np.isfinite(out[77 + 10]) and np.isfinite(out).sum() > 0
    assert sim.observables(raise_on_nan=False)[2]
    sim.upload(rho0)
    sim.evolve(50)
    q = p.copy()
    q.kernel_variant = 2
    ok = CahnHilliard(q, rho0)
    ok.evolve(50)
    assert rel_maxnorm(sim.sync(), ok.sync()) <= 1e-14
    assert not sim.observables()[2]


@pytest.mark.parametrize("dims,N", [(2, 64), (3, 32)])
@pytest.mark.parametrize("scale", ["tiny", "mixed", "zero"])
def test_fixed_point_neighbour_sums_on_extreme_fields(dims, N, scale):
    """The Laplacian's neighbour sums are formed in 64-bit fixed point, with a
    sequential FP64 fallback when every term is below 2^-959 (or zero).  A
    field of that size (tiny), one whose stencils span 1e-150..1e-100 and so
    take both paths (mixed), and an all-zero field: every kernel variant gives
    the same bits, and the oracle's FP64 run agrees to 1e-12 (zero stays zero)."""
    p = config.params(dims, N, "euler", "landau", dt=0.01 if dims == 2 else 0.005, k=1.0, epsilon=0.9)
    rng = np.random.default_rng(11)
    if scale == "tiny":
        rho0 = rng.uniform(-1.0, 1.0, N ** dims) * 1e-295
    elif scale == "mixed":
        rho0 = rng.uniform(-1.0, 1.0, N ** dims) * 10.0 ** rng.uniform(-300, -100, N ** dims)
    else:
        rho0 = np.zeros(N ** dims)
    out = {}
    for v in (1, 2, 5):
        q = p.copy()
        q.kernel_variant = v
        sim = CahnHilliard(q, rho0)
        sim.evolve(20)
        out[v] = sim.sync()
    assert np.array_equal(out[1], out[2])
    ref = oracle.OracleSim(p, rho0)
    ref.step(20)
    if scale == "zero":
        assert not np.any(out[1]) and not np.any(out[5])
    else:
        # variant 5: FP64 sums for the tiny field (its mu unit is below 2^-1000),
        # block fixed point for the mixed one (values 1e200 below the largest drop out)
        assert rel_maxnorm(out[1], ref.rho()) <= TOL and rel_maxnorm(out[5], ref.rho()) <= TOL


@pytest.mark.parametrize("integrator", ["euler", "pseudospectral"])
def test_graph_decompositions_agree(integrator):
    """chgb_step replays cached graphs of 64, 32, ..., 1 steps; any split of the
    same 200 steps (odd counts flip the euler ping-pong parity) gives the same
    bits, and the launch count is the per-step count times the steps."""
    dt = 0.01 if integrator == "euler" else 0.05
    p = config.params(2, 64, integrator, "landau", dt=dt, epsilon=0.9)
    rho0 = config.init_density(2, 64, [0.0], seed=3)
    a = CahnHilliard(p, rho0)
    a.evolve(200)                       # 3 graphs of 64 + one of 8
    b = CahnHilliard(p, rho0)
    for n in (1, 37, 100, 62):
        b.evolve(n)
    c = CahnHilliard(p, rho0)
    for _ in range(200):
        c.evolve(1)
    if integrator == "euler":
        # one or two kernels per step, one kernel per two steps, or one per call (the resident box)
        expected = {1: 200, 2: 400, 3: 100, 4: 1, 5: 201}[a.kernel_variant]
    else:
        expected = 2 + 200 * 2      # initial rho_hat (row + column pass), then two kernels per step
    assert a.launches == expected   # (before sync: rho from rho_hat is one more)
    ra = a.sync()
    assert np.array_equal(ra, b.sync()) and np.array_equal(ra, c.sync())


@pytest.mark.parametrize("model", ["landau", "simple_wertheim", "saleh"])
@pytest.mark.parametrize("dims", [1, 2, 3])
def test_observables_match_oracle(model, dims):
    N = {1: 128, 2: 32, 3: 16}[dims]
    if model == "landau":
        p = config.params(dims, N, "euler", model, dt=0.01, k=1.3, epsilon=0.9)
        rho0 = config.init_density(dims, N, [-0.2], initial_A=0.3, seed=9)
    elif model == "simple_wertheim":
        p = wertheim_params(dims, N, "euler", "constant")
        p.model.density_conversion_factor = 0.125
        rho0 = config.init_density(dims, N, [1e-5], seed=9)
    else:
        p = config.params(dims, N, "euler", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, B3=1e7, delta_AA=1e4,
                          delta_BB=2e4, saleh_valence=(4, 4, 2))
        rho0 = config.init_density(dims, N, [9e-5, 7e-5, 3e-5], seed=5)
    sim = CahnHilliard(p, rho0)
    ref = oracle.OracleSim(p, rho0)
    mass, fe, nan = sim.observables()
    m_ref, _ = ref.average_mass()
    fe_ref, _ = ref.average_free_energy()
    assert not nan
    assert abs(mass - m_ref) <= 1e-13 * np.abs(rho0).mean() * p.dx ** 3
    assert abs(fe - fe_ref) <= 1e-12 * abs(fe_ref)


def test_nan_is_reported_not_fatal():
    p = config.params(2, 32, "euler", "landau", dt=0.01, epsilon=0.9)
    rho0 = config.init_density(2, 32, [0.0], seed=1)
    rho0[77] = np.nan
    sim = CahnHilliard(p, rho0)
    mass, fe, nan = sim.observables(raise_on_nan=False)
    assert nan
    with pytest.raises(abi.ChgbError) as ei:
        sim.observables()
    assert ei.value.code == abi.CHGB_ERR_NAN
    # the context stays usable
    sim.upload(np.zeros(32 * 32))
    sim.evolve(5)
    assert not sim.observables()[2]


def test_upload_with_the_mobility_field():
    """chgb_upload takes the host mobility as CUDAIntegrator::_CPU_GPU does:
    the field the mobility type defines is accepted (and changes nothing),
    any other field is refused with a status code."""
    N = 32
    rho0 = config.init_density(2, N, [0.0], seed=3)
    p = config.params(2, N, "euler_mobility", "landau", dt=0.01, M=0.7, epsilon=0.9)
    a = CahnHilliard(p, rho0)
    b = CahnHilliard(p)
    b.upload(rho0, mobility=np.full(N * N, 0.7))
    a.evolve(20)
    b.evolve(20)
    assert np.array_equal(a.sync(), b.sync())
    bad = np.full(N * N, 0.7)
    bad[5] = 0.71
    with pytest.raises(abi.ChgbError) as ei:
        b.upload(rho0, mobility=bad)
    assert ei.value.code == abi.CHGB_ERR_UNSUPPORTED
    # free-energy mobility: recomputed from rho before every step, so any field is accepted
    pw = wertheim_params(2, N, "euler_mobility", "free_energy")
    rw = config.init_density(2, N, [1e-5], seed=4)
    c = CahnHilliard(pw, rw)
    d = CahnHilliard(pw)
    d.upload(rw, mobility=np.zeros(N * N))
    c.evolve(10)
    d.evolve(10)
    assert np.array_equal(c.sync(), d.sync())


@pytest.mark.parametrize("model", ["landau", "simple_wertheim", "saleh"])
def test_model_device_hooks(model):
    import torch
    lib = abi.load_library()
    if model == "landau":
        p = config.params(2, 32, "euler", model, dt=0.01, epsilon=0.7)
        rho = np.random.default_rng(0).uniform(-1, 1, 1024)
    elif model == "simple_wertheim":
        # f' takes a table-driven logarithm and a Newton-refined reciprocal:
        # uniform densities of the configurations and log-spaced ones over 12 decades
        p = wertheim_params(2, 32, "euler", "constant")
        rng = np.random.default_rng(0)
        rho = np.concatenate([rng.uniform(1e-7, 1e-4, 512), 10.0 ** rng.uniform(-13, -1, 512)])
    else:
        p = config.params(2, 32, "euler", model, dt=1e-6, B2=2190.0, B3=1e7, delta_AA=1e4, delta_BB=2e4)
        rho = np.random.default_rng(0).uniform(1e-6, 1e-4, 3 * 1024)
    bins = 1024
    d_rho = torch.tensor(rho, device="cuda", dtype=torch.float64)
    d_out = torch.zeros_like(d_rho)
    torch.cuda.synchronize()
    abi.check(lib, lib.chgb_der_bulk_free_energy(ctypes.byref(p.model), ctypes.c_void_p(d_rho.data_ptr()),
                                                 ctypes.c_void_p(d_out.data_ptr()), bins, None))
    torch.cuda.synchronize()
    want = oracle.der_bulk_free_energy(p.model, rho, bins)
    got = d_out.cpu().numpy()
    assert rel_maxnorm(got, want) <= 1e-14
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-300)) <= 1e-13   # element by element
    if model == "simple_wertheim":
        abi.check(lib, lib.chgb_set_mobility(ctypes.byref(p.model), ctypes.c_void_p(d_rho.data_ptr()), 2.5,
                                             ctypes.c_void_p(d_out.data_ptr()), bins, None))
        torch.cuda.synchronize()
        assert rel_maxnorm(d_out.cpu().numpy(), oracle.set_mobility(p.model, rho, 2.5)) <= 1e-14
