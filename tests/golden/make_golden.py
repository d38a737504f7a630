"""Generate the golden fixtures of tests/golden/ (run in a checkout that has
the reference sources, after `make -C oracle ref`).

Two kinds of fixture are written:

* reference_goldens.json — the reference's own regression files
  tests/data/reference/landau_{euler,pseudospectral}_{1D,2D,3D}.dat
  (six significant digits, src/utils/Printer.cpp:183-192): the full text of
  the 1D and 2D files and a SHA-1 per line of the 3D files, plus the TOML the
  reference test runs (tests/test_landau.py:27-39, tests/data/simple_landau.toml).
* ref_dumps.npz — full-precision (%.17g-exact, raw FP64) final densities of the
  reference's own CPU integrators on small seeded cases, produced by
  oracle/_ref/ref_harness_<D>D from the TOML texts in CASES, and for the
  Landau cases the reference's pressure field and average pressure.

usage: python tests/golden/make_golden.py /path/to/reference   (or $CHGB_REFERENCE)
       python tests/golden/make_golden.py --driver   (driver_outputs.json.gz)
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "oracle"))
import oracle  # noqa: E402

SIMPLE_SW = """steps = 20
N = 16
dt = 1e-6
initial_density = 5e-5
free_energy = "simple_wertheim"
dx = 10
k = 1e6
seed = 42
integrator = "{integrator}"
[mobility]
type = "{mobility}"
M = 1.0
[wertheim]
valence = 4
B2 = 2190
[wertheim.delta]
T = 300
deltaH = -42200
deltaS = -119.1
salt = 0.5
sticky_size = 6
"""

SALEH = """steps = 20
N = 16
dt = 1e-6
initial_density = 9e-5
free_energy = "saleh"
dx = 10
k = 1e6
seed = 7
integrator = "{integrator}"
[saleh]
valence = [4, 4, 4]
B2 = 2190
B3 = 1e7
[saleh.delta_AA]
T = 293.15
deltaH = -42200
deltaS = -119.1
salt = 0.5
sticky_size = 6
[saleh.delta_BB]
T = 293.15
deltaH = -42400
deltaS = -120.6
salt = 0.5
sticky_size = 6
"""

LANDAU = """steps = 100
N = {N}
dt = {dt}
dx = 1.0
k = {k}
initial_density = {rho0}
free_energy = "landau"
seed = {seed}
integrator = "{integrator}"
[mobility]
M = {M}
[landau]
epsilon = 0.9
[pseudospectral]
S = {S}
use_dealias = {dealias}
"""


GEL_LANDAU = """steps = 100
N = {N}
dt = 0.01
k = 1.0
initial_density = {rho0}
free_energy = "landau"
seed = 2024
integrator = "euler_mobility"
[mobility]
type = "gel"
phi_critical = 0.3
c_0 = 0.1
M_c = 20.0
[landau]
epsilon = 0.9
"""

PSM_LANDAU = """steps = {steps}
N = {N}
dt = {dt}
k = 1.0
initial_density = {rho0}
free_energy = "landau"
seed = 77
integrator = "pseudospectral_mobility"
[pseudospectral]
S = {S}
use_dealias = {dealias}
[mobility]
{mobility}
[landau]
epsilon = 0.9
"""

GEL_MOB = 'type = "gel"\nphi_critical = 0.3\nc_0 = 0.1\nM_c = 20.0'


def gmres(text: str) -> str:
    """The same case with pseudospectral.use_gmres = true and a short restart."""
    return text.replace("use_dealias = ", "use_gmres = true\ngmres_restart = 12\nuse_dealias = ")


GMRES_SW = '[pseudospectral]\nuse_gmres = true\ngmres_tol = 1e-11\n'

REG_SW = SIMPLE_SW.replace('type = "{mobility}"', 'type = "regularised"\nrho_min = 2e-5')


def landau(N, integrator, dt=0.01, k=1.0, rho0=0.0, seed=123456, M=1.0, S=0.0, dealias="false"):
    return LANDAU.format(N=N, integrator=integrator, dt=dt, k=k, rho0=rho0, seed=seed, M=M, S=S, dealias=dealias)


# (name, dims, toml text, steps)
CASES = [
    ("landau_euler_2D_N64", 2, landau(64, "euler"), 100),
    ("landau_euler_2D_N64_offcrit", 2, landau(64, "euler", rho0=-0.3, M=0.7, k=0.8), 100),
    ("landau_euler_1D_N64", 1, landau(64, "euler"), 100),
    ("landau_euler_3D_N16", 3, landau(16, "euler", dt=0.005), 100),
    ("landau_pseudospectral_2D_N64", 2, landau(64, "pseudospectral", dt=0.05), 100),
    ("landau_pseudospectral_2D_N64_S", 2, landau(64, "pseudospectral", dt=0.05, S=0.5, dealias="true",
                                                 rho0=-0.3), 100),
    ("landau_pseudospectral_1D_N64", 1, landau(64, "pseudospectral", dt=0.05, dealias="true"), 100),
    ("landau_pseudospectral_3D_N16", 3, landau(16, "pseudospectral", dt=0.05, dealias="true"), 100),
    ("simple_wertheim_euler_mobility_2D_N16", 2, SIMPLE_SW.format(integrator="euler_mobility",
                                                                    mobility="free_energy"), 20),
    ("simple_wertheim_euler_mobility_3D_N16", 3, SIMPLE_SW.format(integrator="euler_mobility",
                                                                    mobility="free_energy"), 20),
    ("simple_wertheim_euler_2D_N16", 2, SIMPLE_SW.format(integrator="euler", mobility="constant"), 20),
    ("saleh_euler_2D_N16", 2, SALEH.format(integrator="euler"), 20),
    ("saleh_pseudospectral_2D_N16", 2, SALEH.format(integrator="pseudospectral"), 20),
    ("saleh_euler_mobility_3D_N16", 3, SALEH.format(integrator="euler_mobility"), 20),
    ("simple_wertheim_regularised_2D_N16", 2, REG_SW.format(integrator="euler_mobility"), 20),
    ("simple_wertheim_regularised_3D_N16", 3, REG_SW.format(integrator="euler_mobility"), 20),
    ("landau_gel_2D_N32", 2, GEL_LANDAU.format(N=32, rho0=0.0), 100),
    ("landau_gel_1D_N64", 1, GEL_LANDAU.format(N=64, rho0=-0.2), 100),
    ("landau_gel_3D_N16", 3, GEL_LANDAU.format(N=16, rho0=0.1).replace("dt = 0.01", "dt = 0.005"), 100),
    ("landau_psm_gel_2D_N32", 2, PSM_LANDAU.format(steps=100, N=32, dt=0.02, rho0=0.0, S=0.0, dealias="false",
                                                   mobility=GEL_MOB), 100),
    ("landau_psm_gel_2D_N32_S_dealias", 2, PSM_LANDAU.format(steps=100, N=32, dt=0.02, rho0=-0.2, S=0.5,
                                                             dealias="true", mobility=GEL_MOB), 100),
    ("landau_psm_gel_1D_N64", 1, PSM_LANDAU.format(steps=100, N=64, dt=0.02, rho0=0.1, S=0.3, dealias="true",
                                                   mobility=GEL_MOB), 100),
    ("landau_psm_gel_3D_N16", 3, PSM_LANDAU.format(steps=50, N=16, dt=0.02, rho0=0.0, S=0.0, dealias="true",
                                                   mobility=GEL_MOB), 50),
    ("landau_psm_constant_2D_N32", 2, PSM_LANDAU.format(steps=100, N=32, dt=0.05, rho0=0.0, S=0.0,
                                                        dealias="false", mobility="M = 0.8"), 100),
    ("simple_wertheim_psm_free_energy_2D_N16", 2, SIMPLE_SW.format(integrator="pseudospectral_mobility",
                                                                     mobility="free_energy"), 20),
    ("simple_wertheim_psm_regularised_3D_N16", 3, REG_SW.format(integrator="pseudospectral_mobility"), 20),
    ("landau_psm_gmres_gel_2D_N32", 2,
     gmres(PSM_LANDAU.format(steps=30, N=32, dt=0.02, rho0=0.0, S=0.5, dealias="true", mobility=GEL_MOB)), 30),
    ("landau_psm_gmres_gel_2D_N32_nodealias", 2,
     gmres(PSM_LANDAU.format(steps=30, N=32, dt=0.02, rho0=-0.1, S=0.0, dealias="false", mobility=GEL_MOB)), 30),
    ("landau_psm_gmres_gel_1D_N64", 1,
     gmres(PSM_LANDAU.format(steps=40, N=64, dt=0.02, rho0=0.1, S=0.3, dealias="true", mobility=GEL_MOB)), 40),
    ("landau_psm_gmres_gel_3D_N8", 3,
     gmres(PSM_LANDAU.format(steps=10, N=8, dt=0.02, rho0=0.0, S=0.2, dealias="true", mobility=GEL_MOB)), 10),
    ("simple_wertheim_psm_gmres_free_energy_2D_N16", 2,
     SIMPLE_SW.format(integrator="pseudospectral_mobility", mobility="free_energy") + GMRES_SW, 10),
]


def main(ref_root: Path) -> None:
    data_dir = ref_root / "tests" / "data"
    goldens = {"toml": (data_dir / "simple_landau.toml").read_text(), "files": {}}
    for integ in ("euler", "pseudospectral"):
        for d in (1, 2, 3):
            name = f"landau_{integ}_{d}D"
            lines = (data_dir / "reference" / f"{name}.dat").read_text().splitlines()
            entry = {"integrator": integ, "dims": d, "header": lines[0], "n_lines": len(lines)}
            if d < 3:
                entry["text"] = "\n".join(lines)
            else:
                entry["line_sha1"] = [hashlib.sha1(ln.encode()).hexdigest()[:16] for ln in lines]
            goldens["files"][name] = entry
    (HERE / "reference_goldens.json").write_text(json.dumps(goldens, indent=0))

    arrays, meta = {}, []
    work = REPO / "_work" / "golden_tmp"
    for name, dims, text, steps in CASES:
        out = oracle.run_reference(dims, text, steps, work / name)
        arrays[f"{name}__final"] = out["final"]
        if np.ptp(out["mobility"]) != 0.0:
            arrays[f"{name}__mobility"] = out["mobility"]
        arrays[f"{name}__obs"] = np.stack([out["obs_init"], out["obs_final"]])
        if "pressure" in out:
            arrays[f"{name}__pressure"] = out["pressure"]
            arrays[f"{name}__avg_pressure"] = out["average_pressure"]
        # the initial density is regenerated from the seed; its digest pins the drand48 stream
        meta.append({"name": name, "dims": dims, "steps": steps, "toml": text,
                     "init_sha1": hashlib.sha1(out["init"].tobytes()).hexdigest()})
    np.savez_compressed(HERE / "ref_dumps.npz", **arrays)
    (HERE / "ref_dumps.json").write_text(json.dumps(meta, indent=1))
    print(f"wrote {len(meta)} cases")


def reference_root() -> Path:
    """The reference checkout: the first argument that is not an option, else
    $CHGB_REFERENCE."""
    import os
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("CHGB_REFERENCE")
    if not root:
        sys.exit("usage: make_golden.py /path/to/reference   (or set CHGB_REFERENCE)")
    return Path(root)


if __name__ == "__main__" and "--driver" not in sys.argv:
    main(reference_root())


# ---------------------------------------------------------------------------
# Driver fixtures: every output file of the reference's own ch_<D>D program
# (oracle/_ref/ch_<D>D, built from src/main.cpp) on small configurations.
# ---------------------------------------------------------------------------
CADENCE = """steps = {steps}
print_every = {pe}
print_trajectory_every = {pt}
print_last_every = {pl}
"""

DRIVER_CASES = [
    ("landau_euler_2D", 2, CADENCE.format(steps=30, pe=5, pt=10, pl=20) + """N = 32
dt = 0.01
dx = 1.0
k = 1.0
initial_density = 0.0
free_energy = "landau"
seed = 4321
integrator = "euler"
[landau]
epsilon = 0.9
""", {}),
    ("landau_pseudospectral_2D", 2, CADENCE.format(steps=30, pe=5, pt=10, pl=20) + """N = 32
dt = 0.05
k = 1.0
initial_density = -0.3
initial_A = 0.0333333
free_energy = "landau"
seed = 99
integrator = "pseudospectral"
[pseudospectral]
use_dealias = true
[landau]
epsilon = 0.9
""", {}),
    ("landau_euler_3D", 3, CADENCE.format(steps=20, pe=10, pt=10, pl=0) + """N = 16
dt = 0.005
k = 1.0
initial_density = 0.01
free_energy = "landau"
seed = 7
[landau]
T = 0.1
""", {}),
    ("landau_euler_1D", 1, CADENCE.format(steps=40, pe=10, pt=20, pl=20) + """N = 64
dt = 0.01
k = 1.0
initial_density = 0.05
initial_N_peaks = 3
free_energy = "landau"
seed = 11
[landau]
epsilon = 0.7
""", {}),
    ("saleh_euler_2D_scaled", 2, CADENCE.format(steps=10, pe=5, pt=5, pl=10) + """N = 16
dt = 1e-6
dx = 10
k = 1e6
initial_density = 9e-5
free_energy = "saleh"
distance_scaling_factor = 2.0
seed = 3
[saleh]
valence = [4, 4, 4]
B2 = 2190
[saleh.delta_AA]
T = 293.15
deltaH = -42200
deltaS = -119.1
salt = 0.5
sticky_size = 6
[saleh.delta_BB]
T = 293.15
deltaH = -42400
deltaS = -120.6
salt = 0.5
sticky_size = 6
""", {}),
    ("simple_wertheim_mobility_2D", 2, CADENCE.format(steps=20, pe=5, pt=10, pl=10) + """N = 16
dt = 1e-4
dx = 10
k = 1e6
initial_density = 1.107e-5
free_energy = "simple_wertheim"
integrator = "euler_mobility"
distance_scaling_factor = 0.5
seed = 5
[mobility]
type = "free_energy"
M = 1.0
[wertheim]
valence = 4
B2 = 2190
[wertheim.delta]
T = 300
deltaH = -42200
deltaS = -119.1
salt = 0.5
sticky_size = 6
""", {}),
    ("landau_restart_2D", 2, CADENCE.format(steps=20, pe=10, pt=10, pl=10) + """N = 32
dt = 0.01
k = 1.0
load_from = "start.dat"
free_energy = "landau"
seed = 1
[landau]
epsilon = 0.9
""", {"start.dat": "landau_euler_2D/last_0.dat"}),
    ("landau_gel_2D", 2, CADENCE.format(steps=40, pe=10, pt=20, pl=20) + """N = 32
dt = 0.01
k = 1.0
initial_density = 0.0
free_energy = "landau"
integrator = "euler_mobility"
seed = 31
[mobility]
type = "gel"
phi_critical = 0.3
c_0 = 0.1
M_c = 20.0
[landau]
epsilon = 0.9
""", {}),
    ("landau_psm_gel_2D", 2, CADENCE.format(steps=40, pe=10, pt=20, pl=20) + """N = 32
dt = 0.02
k = 1.0
initial_density = -0.1
initial_A = 0.3
free_energy = "landau"
integrator = "pseudospectral_mobility"
seed = 41
[pseudospectral]
S = 0.2
use_dealias = true
[mobility]
type = "gel"
phi_critical = 0.3
c_0 = 0.1
M_c = 20.0
[landau]
epsilon = 0.9
""", {}),
    ("simple_wertheim_regularised_2D", 2, CADENCE.format(steps=20, pe=5, pt=10, pl=10) + """N = 16
dt = 1e-4
dx = 10
k = 1e6
initial_density = 5e-5
free_energy = "simple_wertheim"
integrator = "euler_mobility"
distance_scaling_factor = 0.5
seed = 6
[mobility]
type = "regularised"
M = 1.0
rho_min = 2e-5
[wertheim]
valence = 4
B2 = 2190
[wertheim.delta]
T = 300
deltaH = -42200
deltaS = -119.1
salt = 0.5
sticky_size = 6
""", {}),
    ("landau_pressure_2D", 2, CADENCE.format(steps=30, pe=5, pt=10, pl=20) + """N = 32
dt = 0.01
k = 1.0
initial_density = -0.2
initial_A = 0.3
free_energy = "landau"
seed = 12
integrator = "euler"
[landau]
epsilon = 0.9
[output]
print_pressure = true
print_pressure_every = 10
""", {}),
    ("landau_pressure_log_pseudospectral_2D", 2, """steps = 30
print_every = 5
print_trajectory_strategy = "log"
print_last_every = 10
N = 32
dt = 0.05
k = 1.0
initial_density = 0.0
free_energy = "landau"
seed = 13
integrator = "pseudospectral"
[landau]
epsilon = 0.9
[output]
log_n0 = 4
log_fact = 1.5
print_pressure = true
print_pressure_strategy = "log"
""", {}),
    ("landau_vtk_2D", 2, CADENCE.format(steps=20, pe=10, pt=10, pl=10) + """N = 16
dt = 0.001
dx = 0.5
k = 0.5
initial_density = 0.1
free_energy = "landau"
seed = 14
integrator = "euler"
[landau]
epsilon = 0.9
[output]
print_vtk = true
trajectory_path = "."
print_pressure = true
print_pressure_every = 10
""", {}),
    ("landau_vtk_3D", 3, CADENCE.format(steps=10, pe=5, pt=5, pl=10) + """N = 8
dt = 0.005
k = 1.0
initial_density = 0.0
free_energy = "landau"
seed = 15
integrator = "euler"
[landau]
epsilon = 0.9
[output]
print_vtk = true
trajectory_path = "."
""", {}),
    ("landau_restart_3D", 3, CADENCE.format(steps=10, pe=5, pt=5, pl=10) + """N = 16
dt = 0.005
k = 1.0
load_from = "start.dat"
free_energy = "landau"
seed = 1
[landau]
T = 0.1
""", {"start.dat": "landau_euler_3D/last_0.dat"}),
    ("saleh_pressure_2D", 2, CADENCE.format(steps=10, pe=5, pt=5, pl=10) + """N = 16
dt = 1e-6
dx = 10
k = 1e6
initial_density = 9e-5
free_energy = "saleh"
seed = 16
[saleh]
valence = [4, 4, 4]
B2 = 2190
delta_AA = 1e4
delta_BB = 2e4
[output]
print_pressure = true
print_pressure_every = 5
""", {}),
]


def make_driver_fixtures(work: Path) -> dict:
    import shutil
    import subprocess
    out = {}
    for name, dims, text, inputs in DRIVER_CASES:
        d = work / "driver" / name
        if d.exists():
            shutil.rmtree(d)
        d.mkdir(parents=True)
        (d / "input.toml").write_text(text)
        files_in = {}
        for dst, src in inputs.items():
            content = (work / "driver" / src).read_text()
            (d / dst).write_text(content)
            files_in[dst] = content
        # a model without a pressure makes the reference stop (exit code 1) after the init_ files
        r = subprocess.run([str(REPO / "oracle" / "_ref" / f"ch_{dims}D"), "input.toml"], cwd=d,
                           capture_output=True)
        files = {p.name: p.read_text() for p in sorted(d.iterdir())
                 if p.name not in ("input.toml",) and p.name not in inputs}
        out[name] = {"dims": dims, "toml": text, "inputs": files_in, "outputs": files, "rc": r.returncode}
    return out


def main_driver() -> None:
    work = REPO / "_work" / "golden_tmp"
    fixtures = make_driver_fixtures(work)
    import gzip
    with gzip.open(HERE / "driver_outputs.json.gz", "wt") as f:
        json.dump(fixtures, f)
    print(f"wrote {len(fixtures)} driver cases")


if __name__ == "__main__" and "--driver" in sys.argv:
    main_driver()
