"""The reference-side drop-in integrator (cahn-hilliard_gb300/host/GB300Integrator.h)
compiled against the reference's own headers and linked with libchgb.so
(`make -C oracle dropin`, which needs the reference sources: skipped where they
are absent).

* It builds, and its chgb_params -- the reference's TOML keys scaled as the
  reference's constructors scale them -- equal the ones the drop-in driver
  ch_<D>D builds (itself checked against the Python mirror) on every driver
  fixture configuration.
* Run without a GPU it stops in chgb_create through the reference's
  critical(), naming the integrator: the reference's object did call into the
  engine.  The reference's own validate() still rejects a non-constant
  mobility with `euler` before the engine is reached.
"""
import gzip
import json
import subprocess

import pytest

from conftest import GOLDEN, REPO, gpu_available

REF = REPO / "oracle" / "_ref"
LIB = REPO / "cahn-hilliard_gb300" / "lib"

KEYS = ["dims", "N", "integrator", "mobility_type", "dt", "dx", "k", "M", "splitting_S", "use_dealias", "kind",
        "n_species", "epsilon", "valence", "saleh_valence", "B2", "B3", "delta", "regularisation_delta", "delta_AA",
        "delta_BB", "density_conversion_factor", "rho_min", "gel"]


@pytest.fixture(scope="module")
def dropin():
    if not (REF / "ch_2D").exists() or not (LIB / "libchgb.so").exists():
        pytest.skip("reference CPU build (oracle/_ref) or libchgb.so not present")
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "dropin"], check=True, capture_output=True)
    return {d: REF / f"gb300_dropin_{d}D" for d in (1, 2, 3)}


def _json_line(stdout):
    return json.loads([ln for ln in stdout.splitlines() if ln.startswith("{")][-1])


def test_dropin_params_match_the_driver(dropin, tmp_path):
    cases = json.load(gzip.open(GOLDEN / "driver_outputs.json.gz", "rt"))
    n = 0
    for name, case in cases.items():
        if "load_from" in case["toml"]:
            continue
        cfg = tmp_path / f"{name}.toml"
        cfg.write_text(case["toml"])
        dims = case["dims"]
        got = _json_line(subprocess.run([str(dropin[dims]), "--print-params", str(cfg)], capture_output=True,
                                        text=True, check=True).stdout)
        want = _json_line(subprocess.run([str(LIB / f"ch_{dims}D"), "--print-params", str(cfg)],
                                         capture_output=True, text=True, check=True).stdout)
        for key in KEYS:
            assert got[key] == want[key], (name, key, got[key], want[key])
        n += 1
    assert n >= 12


def test_dropin_calls_into_the_engine(dropin, tmp_path):
    if gpu_available():
        pytest.skip("with a GPU the run would succeed; this checks the path to chgb_create without one")
    cfg = tmp_path / "in.toml"
    cfg.write_text('steps = 10\nN = 32\ndt = 0.01\nk = 1.0\ninitial_density = 0.0\nfree_energy = "landau"\n'
                   'seed = 3\nintegrator = "euler"\n[landau]\nepsilon = 0.9\n')
    r = subprocess.run([str(dropin[2]), str(cfg), "10", str(tmp_path / "out")], capture_output=True, text=True)
    out = r.stdout + r.stderr
    assert r.returncode == 1
    assert "GB300Integrator" in out and "critical" in out
    # the reference's factory and validate() run before the swap, as in the reference
    cfg.write_text(cfg.read_text().replace("[landau]", '[mobility]\ntype = "free_energy"\n[landau]'))
    r = subprocess.run([str(dropin[2]), str(cfg), "10", str(tmp_path / "out")], capture_output=True, text=True)
    assert r.returncode == 1 and "only supports constant mobility" in r.stdout + r.stderr
