import json
import sys
import tomllib
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
for p in (REPO / "cahn-hilliard_gb300", REPO / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def rel_maxnorm(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="session")
def ref_dumps():
    meta = json.loads((GOLDEN / "ref_dumps.json").read_text())
    data = np.load(GOLDEN / "ref_dumps.npz")
    cases = []
    for m in meta:
        c = dict(m)
        c["cfg"] = tomllib.loads(m["toml"])
        c["final"] = data[f"{m['name']}__final"]
        c["obs"] = data[f"{m['name']}__obs"]
        key = f"{m['name']}__mobility"
        c["mobility"] = data[key] if key in data.files else None
        key = f"{m['name']}__pressure"       # Landau cases: the reference's pressure() and average_pressure()
        c["pressure"] = data[key] if key in data.files else None
        c["avg_pressure"] = data[f"{m['name']}__avg_pressure"] if key in data.files else None
        cases.append(c)
    return cases


@pytest.fixture(scope="session")
def ref_goldens():
    return json.loads((GOLDEN / "reference_goldens.json").read_text())


def setup_case(case):
    """Params + initial density of a golden case (reference TOML keys)."""
    from chgb import config
    st = config.setup_from_config(case["cfg"])
    p = st.params
    p.dims = case["dims"]
    rho0 = config.init_density(p.dims, p.N, st.initial_density, st.initial_A, st.initial_N_peaks,
                               st.user_to_internal, st.seed)
    return st, p, rho0


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
