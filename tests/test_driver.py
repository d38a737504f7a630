"""The drop-in driver ch_<D>D (C++ host over the C ABI) against the reference's
own ch_<D>D program: same TOML in, same files out (init_/last_/traj_,
energy.dat), and the reference's regression test (tests/test_landau.py of the
reference: last_0.dat after 100 steps vs its golden files, mass conservation).
"""
import gzip
import hashlib
import json
import subprocess
import tomllib
from pathlib import Path

import numpy as np
import pytest

from chgb import config
from conftest import GOLDEN, REPO

LIB = REPO / "cahn-hilliard_gb300" / "lib"


def driver(dims):
    exe = LIB / f"ch_{dims}D"
    if not exe.exists():
        pytest.skip("driver not built")
    return exe


@pytest.fixture(scope="module")
def driver_cases():
    return json.load(gzip.open(GOLDEN / "driver_outputs.json.gz", "rt"))


# ---------------------------------------------------------------- CPU ------
def test_print_params_matches_python_config(driver_cases, tmp_path):
    """The C++ TOML handling (keys, defaults, Delta, unit scaling, seeded
    initial density) agrees with the Python mirror, without a GPU."""
    for name, case in driver_cases.items():
        if "load_from" in case["toml"]:
            continue
        cfg_path = tmp_path / f"{name}.toml"
        cfg_path.write_text(case["toml"])
        r = subprocess.run([str(driver(case["dims"])), "--print-params", str(cfg_path)], capture_output=True,
                           text=True, check=True)
        got = json.loads(r.stdout)
        st = config.setup_from_config(tomllib.loads(case["toml"]))
        p = st.params
        m = p.model
        assert got["N"] == p.N and got["integrator"] == p.integrator and got["mobility_type"] == p.mobility_type
        for key in ("dt", "dx", "M", "splitting_S"):
            assert got[key] == getattr(p, key), (name, key)
        assert got["k"][:m.n_species] == list(p.k)[:m.n_species]
        for key in ("epsilon", "B2", "B3", "delta", "regularisation_delta", "delta_AA", "delta_BB",
                    "density_conversion_factor"):
            assert got[key] == pytest.approx(getattr(m, key), rel=1e-15, abs=0), (name, key)
        assert got["steps"] == st.steps
        assert got["rho_min"] == p.rho_min
        assert got["gel"] == pytest.approx([p.gel_phi_critical, p.gel_c0, p.gel_M_c, p.gel_beta_delta_F],
                                           rel=1e-15, abs=0)
        rho0 = config.init_density(case["dims"], p.N, st.initial_density, st.initial_A, st.initial_N_peaks,
                                   st.user_to_internal, st.seed)
        assert got["rho_sum"] == pytest.approx(rho0.sum(), rel=1e-13, abs=1e-15)


def test_print_params_rejects_like_the_reference(tmp_path):
    bad = tmp_path / "bad.toml"
    bad.write_text('steps = 1\nN = 48\ndt = 0.1\nk = 1.0\ninitial_density = 0.0\nfree_energy = "landau"\n'
                   '[landau]\nepsilon = 0.9\n')
    r = subprocess.run([str(driver(2)), "--print-params", str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "power of 2" in r.stderr
    bad.write_text('steps = 1\nN = 16\ndt = 0.1\nk = 1\ninitial_density = 0.0\nfree_energy = "landau"\n'
                   '[landau]\nepsilon = 0.9\n')
    r = subprocess.run([str(driver(2)), "--print-params", str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "'k'" in r.stderr


# ---------------------------------------------------------------- GPU ------
def _tokens(text):
    return [ln.split() for ln in text.splitlines()]


def compare_files(name, got, want, rel):
    g, w = _tokens(got), _tokens(want)
    assert len(g) == len(w), f"{name}: {len(g)} lines vs {len(w)}"
    ntok = ndiff = 0
    for lg, lw in zip(g, w):
        assert len(lg) == len(lw), name
        for a, b in zip(lg, lw):
            ntok += 1
            if a == b:
                continue
            ndiff += 1
            fa, fb = float(a), float(b)
            assert abs(fa - fb) <= rel * max(abs(fa), abs(fb)) + 1e-300, f"{name}: {a} vs {b}"
    # byte for byte: on GB300 every file of every fixture is the reference
    # program's (the tolerance above only words the message of a failure)
    assert ndiff == 0, f"{name}: {ndiff} of {ntok} tokens differ"


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["landau_euler_2D", "landau_pseudospectral_2D", "landau_euler_3D",
                                  "landau_euler_1D", "saleh_euler_2D_scaled", "simple_wertheim_mobility_2D",
                                  "landau_restart_2D", "landau_gel_2D", "simple_wertheim_regularised_2D",
                                  "landau_psm_gel_2D", "landau_pressure_2D", "landau_pressure_log_pseudospectral_2D",
                                  "landau_vtk_2D", "landau_vtk_3D", "landau_restart_3D", "saleh_pressure_2D"])
def test_driver_outputs_match_reference_program(driver_cases, name, tmp_path):
    """Every file of the reference program's run, byte for byte, and its exit code: pressure
    (linear and log cadence, the energy.dat column, snapshots, and trajectories
    that hold the density as the reference writes them), VTK output in 2D and
    3D, the log trajectory strategy, 2D and 3D restarts (the reference reads N
    lines of a 3D file), and a model without a pressure stopping after the
    init_ files."""
    case = driver_cases[name]
    (tmp_path / "input.toml").write_text(case["toml"])
    for fn, content in case["inputs"].items():
        (tmp_path / fn).write_text(content)
    r = subprocess.run([str(driver(case["dims"])), "input.toml"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == case.get("rc", 0), r.stderr
    if case.get("rc", 0):
        assert "pressure coupling" in r.stderr
    produced = {p.name for p in tmp_path.iterdir()} - {"input.toml"} - set(case["inputs"])
    assert produced == set(case["outputs"]), produced ^ set(case["outputs"])
    for fn, want in case["outputs"].items():
        got = (tmp_path / fn).read_text()
        if fn == "energy.dat":
            compare_files(fn, got, want, rel=5e-7)
            # stdout carries the same lines
            assert r.stdout.strip().splitlines() == got.strip().splitlines()
        else:
            compare_files(fn, got, want, rel=2e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["euler", "pseudospectral"])
@pytest.mark.parametrize("dims", [1, 2, 3])
def test_reference_regression_test(ref_goldens, integrator, dims, tmp_path):
    """The reference's tests/test_landau.py run against ch_<D>D: the golden
    last_0.dat (six digits, compared at rtol 1e-12 there) and mass conservation."""
    text = f'\nintegrator = "{integrator}"\n' + ref_goldens["toml"]
    (tmp_path / "simple_landau.toml").write_text(text)
    subprocess.run([str(driver(dims)), "simple_landau.toml"], cwd=tmp_path, check=True, capture_output=True,
                   timeout=300)
    entry = ref_goldens["files"][f"landau_{integrator}_{dims}D"]
    lines = (tmp_path / "last_0.dat").read_text().splitlines()[1:]
    if "text" in entry:
        want = entry["text"].split("\n")[1:]
        got = [ln for ln in lines]
        assert [ln.rstrip() for ln in got] == [ln.rstrip() for ln in want]
    else:
        digests = [hashlib.sha1(ln.encode()).hexdigest()[:16] for ln in lines]
        assert digests == entry["line_sha1"][1:]
    phi0 = np.loadtxt(tmp_path / "init_0.dat")
    phi1 = np.loadtxt(tmp_path / "last_0.dat")
    assert abs(phi0.sum() - phi1.sum()) < 1e-4


@pytest.mark.gpu
def test_full_precision_restart_3d(tmp_path):
    """3D with `load_from_full_3d = true` (a key the reference does not have)
    and 17-digit files: 20 steps + a restart reading all N*N lines + 20 steps
    equal 40 straight steps to the bit.  Without the flag the reference's N-line
    reading is kept (the driver fixture landau_restart_3D)."""
    base = ('integrator = "euler"\nN = 16\ndt = 0.005\nk = 1.0\nfree_energy = "landau"\n'
            'initial_density = 0.0\nseed = 8\nprint_every = 10\nprint_trajectory_every = 0\n'
            '[landau]\nepsilon = 0.9\n[output]\nfull_precision = true\n')
    for name, toml in {"a": "steps = 20\nprint_last_every = 20\n" + base,
                       "c": "steps = 40\nprint_last_every = 40\n" + base}.items():
        d = tmp_path / name
        d.mkdir()
        (d / "input.toml").write_text(toml)
        subprocess.run([str(driver(3)), "input.toml"], cwd=d, check=True, capture_output=True, timeout=300)
    b = tmp_path / "b"
    b.mkdir()
    restart = (f'load_from = "{tmp_path / "a" / "last_0.dat"}"\nload_from_full_3d = true\nsteps = 20\n'
               'print_last_every = 20\n' + base.replace("initial_density = 0.0\n", ""))
    (b / "input.toml").write_text(restart)
    subprocess.run([str(driver(3)), "input.toml"], cwd=b, check=True, capture_output=True, timeout=300)
    g = np.array([float(x) for ln in (b / "last_0.dat").read_text().splitlines()[1:] for x in ln.split()])
    w = np.array([float(x) for ln in (tmp_path / "c" / "last_0.dat").read_text().splitlines()[1:] for x in ln.split()])
    assert g.size == w.size == 16 ** 3
    assert np.array_equal(g, w)


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["euler", "pseudospectral"])
def test_full_precision_restart(integrator, tmp_path):
    """`output.full_precision = true` writes 17 digits, so 100 steps + a
    load_from restart + 100 steps equal 200 straight steps: to the bit for the
    explicit step, to 1e-12 for the pseudospectral one (the restart redoes the
    forward transform of the real field)."""
    dt = 0.01 if integrator == "euler" else 0.05
    base = (f'integrator = "{integrator}"\nN = 64\ndt = {dt}\nk = 1.0\nfree_energy = "landau"\n'
            'initial_density = 0.0\nseed = 7\nprint_every = 50\nprint_trajectory_every = 0\n'
            '[landau]\nepsilon = 0.9\n[output]\nfull_precision = true\n')
    runs = {"a": "steps = 100\nprint_last_every = 100\n" + base,
            "c": "steps = 200\nprint_last_every = 200\n" + base}
    for name, toml in runs.items():
        d = tmp_path / name
        d.mkdir()
        (d / "input.toml").write_text(toml)
        subprocess.run([str(driver(2)), "input.toml"], cwd=d, check=True, capture_output=True, timeout=300)
    b = tmp_path / "b"
    b.mkdir()
    restart = (f'load_from = "{tmp_path / "a" / "last_0.dat"}"\nsteps = 100\nprint_last_every = 100\n'
               + base.replace("initial_density = 0.0\n", ""))
    (b / "input.toml").write_text(restart)
    subprocess.run([str(driver(2)), "input.toml"], cwd=b, check=True, capture_output=True, timeout=300)
    got = (b / "last_0.dat").read_text().splitlines()
    want = (tmp_path / "c" / "last_0.dat").read_text().splitlines()
    # the final last_ header carries `steps`, not the restart's absolute step,
    # as the reference's Manager::run writes it (src/main.cpp:133)
    assert got[0].startswith("# step = 100,") and want[0].startswith("# step = 200,")
    g = np.array([float(x) for ln in got[1:] for x in ln.split()])
    w = np.array([float(x) for ln in want[1:] for x in ln.split()])
    assert g.size == w.size == 64 * 64
    if integrator == "euler":
        assert np.array_equal(g, w)
    else:
        assert np.max(np.abs(g - w)) <= 1e-12 * np.max(np.abs(w))
