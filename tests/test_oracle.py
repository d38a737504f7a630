"""CPU tests of the oracle: pinned against the reference's golden files and
against full-precision dumps of the reference's own CPU integrators."""
import hashlib
import math

import numpy as np
import pytest

import oracle
from chgb import config
from conftest import rel_maxnorm, setup_case


def fmt_native_lines(rho, N, dims):
    """Data lines of the reference's native writer (src/utils/Printer.cpp:183-192):
    default ostream precision (%g), a space after every value, a newline every
    N values in 2D/3D and after every value in 1D."""
    per_line = N if dims >= 2 else 1
    vals = ["%g " % v for v in rho]
    return ["".join(vals[i:i + per_line]) for i in range(0, len(vals), per_line)]


def run_golden_config(ref_goldens, name):
    entry = ref_goldens["files"][name]
    text = f'\nintegrator = "{entry["integrator"]}"\n' + ref_goldens["toml"]
    import tomllib
    st = config.setup_from_config(tomllib.loads(text))
    p = st.params
    p.dims = entry["dims"]
    rho0 = config.init_density(p.dims, p.N, st.initial_density, st.initial_A, st.initial_N_peaks,
                               st.user_to_internal, st.seed)
    sim = oracle.OracleSim(p, rho0)
    sim.step(st.steps)
    return entry, sim.rho(), p


@pytest.mark.parametrize("name", [f"landau_{i}_{d}D" for i in ("euler", "pseudospectral") for d in (1, 2, 3)])
def test_oracle_reproduces_reference_golden_files(ref_goldens, name):
    """tests/test_landau.py of the reference: last_0.dat after 100 steps, six digits."""
    entry, rho, p = run_golden_config(ref_goldens, name)
    lines = fmt_native_lines(rho, p.N, p.dims)
    assert len(lines) == entry["n_lines"] - 1
    if "text" in entry:
        want = entry["text"].split("\n")[1:]
        assert lines == want
    else:
        got = [hashlib.sha1(ln.encode()).hexdigest()[:16] for ln in lines]
        assert got == entry["line_sha1"][1:]


def test_golden_mass_conservation(ref_goldens):
    """The reference's test_mass_conservation bound (|sum before - sum after| < 1e-4)."""
    for name in ("landau_euler_2D", "landau_pseudospectral_2D"):
        entry, rho, p = run_golden_config(ref_goldens, name)
        rho0 = config.init_density(2, 64, [0.01], 1e-2, 0, 1.0, 123456)
        assert abs(rho0.sum() - rho.sum()) < 1e-12 * abs(rho0).sum() * 100


def test_init_density_matches_reference_drand48(ref_dumps):
    for case in ref_dumps:
        st, p, rho0 = setup_case(case)
        assert hashlib.sha1(rho0.tobytes()).hexdigest() == case["init_sha1"], case["name"]
        c_rho0 = oracle.init_density(p.dims, p.N, st.initial_density, st.initial_A, st.initial_N_peaks,
                                     st.user_to_internal, st.seed)
        assert np.array_equal(c_rho0, rho0)


def test_oracle_matches_reference_dumps(ref_dumps):
    for case in ref_dumps:
        st, p, rho0 = setup_case(case)
        sim = oracle.OracleSim(p, rho0)
        sim.step(case["steps"])
        err = rel_maxnorm(sim.rho(), case["final"])
        assert err <= 1e-13, (case["name"], err)
        if case["mobility"] is not None:
            assert rel_maxnorm(sim.mobility(), case["mobility"]) <= 1e-13
        mass, nan1 = sim.average_mass()
        fe, nan2 = sim.average_free_energy()
        assert not nan1 and not nan2
        m_ref, fe_ref = case["obs"][1]
        assert abs(mass - m_ref) <= 1e-13 * abs(m_ref) + 1e-18
        assert abs(fe - fe_ref) <= 1e-11 * abs(fe_ref) + 1e-18, (case["name"], fe, fe_ref)


def test_oracle_pressure_matches_reference_dumps(ref_dumps):
    """The oracle's pressure field and average pressure against the
    reference's own CahnHilliard::pressure() / average_pressure() on every
    Landau case (initial state and after the run), and the reference's
    refusal for the other models."""
    n = 0
    for case in ref_dumps:
        st, p, rho0 = setup_case(case)
        sim = oracle.OracleSim(p, rho0)
        if case["pressure"] is None:
            with pytest.raises(ValueError, match="pressure coupling"):
                sim.average_pressure()
            continue
        n += 1
        assert abs(sim.average_pressure() - case["avg_pressure"][0]) <= 1e-12 * abs(case["avg_pressure"][0])
        sim.step(case["steps"])
        assert rel_maxnorm(sim.pressure(), case["pressure"]) <= 1e-13, case["name"]
        got = sim.average_pressure()
        assert abs(got - case["avg_pressure"][1]) <= 1e-12 * abs(case["avg_pressure"][1]), (case["name"], got)
    assert n >= 10


@pytest.mark.parametrize("shape", [(64,), (8,), (32, 64), (16, 16), (8, 16, 32), (4, 4, 4)])
def test_oracle_fft_matches_numpy(shape):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape)
    h = oracle.rfftn(a)
    want = np.fft.rfftn(a)
    assert np.max(np.abs(h - want)) <= 1e-13 * np.max(np.abs(want))
    back = oracle.irfftn(want, shape) / a.size
    assert np.max(np.abs(back - a)) <= 1e-14 * np.max(np.abs(a))


def test_drand48_stream_known_values():
    # srand48(0) then drand48(): X1 = (0x5DEECE66D * 0x330E + 0xB) mod 2^48
    x = (0x5DEECE66D * 0x330E + 0xB) & ((1 << 48) - 1)
    v = config.drand48_stream(0, 5000)
    assert v[0] == x / 2.0 ** 48
    # the vectorised jump agrees with the sequential recurrence across block edges
    seq = []
    x = ((123456 & 0xFFFFFFFF) << 16) | 0x330E
    for _ in range(5000):
        x = (0x5DEECE66D * x + 0xB) & ((1 << 48) - 1)
        seq.append(x / 2.0 ** 48)
    assert np.array_equal(config.drand48_stream(123456, 5000), np.array(seq))


def test_delta_from_thermodynamics():
    node = {"T": 300, "deltaH": -42200, "deltaS": -119.1, "salt": 0.5, "sticky_size": 6}
    d = config.delta_value(node, "wertheim.delta")
    dS_salt = 0.368 * 5 * math.log(0.5)
    dG = -42200 - 300 * (-119.1 + dS_salt)
    assert d == pytest.approx(1.6606 * math.exp(-dG / (1.9872036 * 300)), rel=1e-15)
    assert config.delta_value(12.5, "x") == 12.5
    assert config.delta_value({"value": 3.0}, "x") == 3.0


def test_config_rejections():
    base = {"steps": 10, "N": 64, "dt": 0.01, "k": 1.0, "free_energy": "landau", "landau": {"epsilon": 0.9},
            "initial_density": 0.0}
    config.setup_from_config(base)
    with pytest.raises(config.ConfigError, match="power of 2"):
        config.setup_from_config({**base, "N": 48})
    with pytest.raises(config.ConfigError, match="distance_scaling_factor"):
        config.setup_from_config({**base, "distance_scaling_factor": 2.0})
    with pytest.raises(config.ConfigError, match="constant mobility"):
        config.setup_from_config({**base, "mobility": {"type": "free_energy"}})
    with pytest.raises(config.ConfigError, match="mobility coupling"):
        config.setup_from_config({**base, "integrator": "euler_mobility", "mobility": {"type": "free_energy"}})
    with pytest.raises(config.ConfigError, match="initial_density"):
        config.setup_from_config({k: v for k, v in base.items() if k != "initial_density"})
    # k given as an integer is not a floating-point node: the reference rejects it
    with pytest.raises(config.ConfigError):
        config.setup_from_config({**base, "k": 1})
    st = config.setup_from_config({**base, "landau": {"T": 0.25}})
    assert st.params.model.epsilon == 0.75


def test_unit_scaling_simple_wertheim():
    cfg = {"steps": 1, "N": 16, "dt": 1e-6, "dx": 10.0, "k": 1e6, "free_energy": "simple_wertheim",
           "initial_density": 5e-5, "distance_scaling_factor": 2.0,
           "wertheim": {"valence": 4, "B2": 2190.0, "delta": 100.0, "regularisation_delta": 1e-8},
           "mobility": {"type": "free_energy", "M": 3.0}, "integrator": "euler_mobility"}
    st = config.setup_from_config(cfg)
    u = 0.5
    p = st.params
    assert p.dx == 10.0 * u
    assert p.k[0] == 1e6 * u ** 5
    assert p.M == 3.0 / u
    assert p.model.B2 == 2190.0 * u ** 3
    assert p.model.delta == 100.0 * u ** 3
    assert p.model.regularisation_delta == 1e-8 / u ** 3
    assert p.model.density_conversion_factor == u ** 3
