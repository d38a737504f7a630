"""chgb_observables_noalloc: the observables entry point for callers that
cannot allocate device memory when they need the mass and free energy (their
pool already owns HBM, or their loop cannot pay for cudaMalloc/cudaFree).

It is checked through the C ABI against the existing entry point
chgb_observables on two calls in a row (the second call reuses the library's
fixed scratch array), within the tolerances of the other observables tests:
the two sum in different block orders, so they agree to round-off, not to the
bit.  Cases: Landau 2D, Saleh 3D, simple_wertheim 1D on a side stream, and a
call made in a fresh process before any handle exists (no scratch address
looked up yet, no logarithm table on the device).  The size checks run on the
CPU: they reject before any device access.  This file is collected last so
that a run stopping at the first failure has already run every other test; it
also passes alone in a fresh process.
"""
import ctypes
import json
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

from chgb import abi, config

PKG = Path(__file__).resolve().parent.parent / "cahn-hilliard_gb300"


def _noalloc(lib, p, d_rho_ptr, stream=None):
    import torch
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    s = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    code = lib.chgb_observables_noalloc(ctypes.byref(p), ctypes.c_void_p(d_rho_ptr), ctypes.c_void_p(out.data_ptr()),
                                        s)
    abi.check(lib, code)
    if stream is not None:
        stream.synchronize()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _wertheim_params(dims, N):
    return config.params(dims, N, "euler", "simple_wertheim", dt=1e-4, dx=10.0, k=1e6, M=1.0, valence=4, B2=2190.0,
                         delta=config.delta_value({"T": 300, "deltaH": -42200, "deltaS": -119.1, "salt": 0.5,
                                                   "sticky_size": 6}, "d"))


def _field(case):
    from chgb.sim import CahnHilliard
    if case == "landau2d":
        p = config.params(2, 128, "euler", "landau", dt=0.01, k=1.0, epsilon=0.9)
        rho0 = config.init_density(2, 128, [-0.2], initial_A=0.3, seed=31)
        steps = 30
    elif case == "saleh3d":
        p = config.params(3, 16, "euler", "saleh", dt=1e-6, dx=10.0, k=1e6, B2=2190.0, B3=1e7, delta_AA=1e4,
                          delta_BB=2e4, saleh_valence=(4, 4, 2))
        rho0 = config.init_density(3, 16, [9e-5, 7e-5, 3e-5], seed=5)
        steps = 10
    else:                                             # simple_wertheim 1D
        p = _wertheim_params(1, 4096)
        rho0 = config.init_density(1, 4096, [1.107e-5], seed=8)
        steps = 20
    sim = CahnHilliard(p, rho0)
    sim.evolve(steps)
    return p, sim, rho0


def _close(got, mass, fe, rho0, dx):
    return (abs(got[0] - mass) <= 1e-13 * np.abs(rho0).mean() * dx ** 3 + 1e-300
            and abs(got[1] - fe) <= 1e-12 * abs(fe))


@pytest.mark.gpu
def test_noalloc_matches_chgb_observables_two_calls():
    lib = abi.load_library()
    results = []
    for case in ("landau2d", "saleh3d"):           # two calls in a row, different fields
        p, sim, rho0 = _field(case)
        mass, fe, nan = sim.observables()           # the existing entry point
        sim.synchronize()
        got = _noalloc(lib, p, sim.device_rho())
        results.append((got, mass, fe))
        assert not nan
        assert _close(got, mass, fe, rho0, p.dx), (case, got, mass, fe)
        sim.close()
    # the first field again: the scratch keeps the last call's contents, which must not leak in
    p, sim, rho0 = _field("landau2d")
    sim.synchronize()
    again = _noalloc(lib, p, sim.device_rho())
    assert np.array_equal(again, results[0][0])
    sim.close()


@pytest.mark.gpu
def test_noalloc_simple_wertheim_1d_on_a_side_stream():
    import torch
    lib = abi.load_library()
    p, sim, rho0 = _field("wertheim1d")
    mass, fe, nan = sim.observables()
    sim.synchronize()
    side = torch.cuda.Stream()
    got = [_noalloc(lib, p, sim.device_rho(), stream=side) for _ in range(2)]
    assert not nan
    assert np.array_equal(got[0], got[1])
    assert _close(got[0], mass, fe, rho0, p.dx), (got[0], mass, fe)
    sim.close()


_FRESH = textwrap.dedent("""
    import ctypes, json, sys
    sys.path.insert(0, {pkg!r})
    sys.path.insert(0, {tests!r})
    import torch
    from chgb import abi, config
    from chgb.sim import CahnHilliard
    from test_zz_no_alloc import _wertheim_params
    lib = abi.load_library()
    p = _wertheim_params(2, 64)
    rho0 = config.init_density(2, 64, [1.107e-5], seed=9)
    d_rho = torch.from_numpy(rho0).cuda()
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    first = []
    for _ in range(2):       # before any handle: no scratch address yet, no logarithm table
        code = lib.chgb_observables_noalloc(ctypes.byref(p), ctypes.c_void_p(d_rho.data_ptr()),
                                            ctypes.c_void_p(out.data_ptr()), None)
        abi.check(lib, code)
        torch.cuda.synchronize()
        first.append(out.cpu().tolist())
    sim = CahnHilliard(p, rho0)
    mass, fe, nan = sim.observables()
    sim.close()
    print(json.dumps({{"first": first, "mass": mass, "fe": fe, "nan": bool(nan),
                      "scale": float(abs(rho0).mean()), "dx": p.dx}}))
""")


@pytest.mark.gpu
def test_noalloc_first_call_in_a_fresh_process(tmp_path):
    script = tmp_path / "fresh.py"
    script.write_text(_FRESH.format(pkg=str(PKG), tests=str(Path(__file__).resolve().parent)))
    r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert not res["nan"]
    assert res["first"][0] == res["first"][1]
    assert _close(res["first"][0], res["mass"], res["fe"], np.array([res["scale"]]), res["dx"]), res


@pytest.mark.parametrize("dims,N,what", [
    (3, 512, "exceeds the no-allocation scratch"),     # 134 M cells > 16.7 M
    (2, 8192, "exceeds the no-allocation scratch"),    # 67 M cells
    (3, 1 << 21, "at most 1024"),                      # N^3 would overflow 64 bits
    (3, 1 << 22, "at most 1024"),
    (2, 1 << 15, "at most 16384"),
    (1, 1 << 25, "at most 16777216"),
])
def test_noalloc_rejects_sizes_on_the_host(dims, N, what):
    lib = abi.load_library()
    p = config.params(3, 64, "euler", "landau", dt=0.01, epsilon=0.9)
    p.dims, p.N = dims, N
    dummy = ctypes.c_void_p(256)        # rejected before any device access
    code = lib.chgb_observables_noalloc(ctypes.byref(p), dummy, dummy, None)
    assert code == abi.CHGB_ERR_INVALID
    assert what in lib.chgb_last_error(None).decode()
