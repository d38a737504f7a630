"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline leg of bench.py, always as the checker or the timed CPU
reference -- never as the product path.
"""
from __future__ import annotations

import ctypes
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(REPO / "cahn-hilliard_gb300"))
from chgb import abi  # noqa: E402  (parameter structs shared with the C ABI)

LIB_PATH = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

_lib = None
_D = ctypes.POINTER(ctypes.c_double)


def build() -> None:
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.och_create.restype = ctypes.c_void_p
        L.och_create.argtypes = [ctypes.POINTER(abi.Params), _D]
        L.och_destroy.argtypes = [ctypes.c_void_p]
        L.och_step.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.och_get_rho.argtypes = [ctypes.c_void_p, _D]
        L.och_get_mobility.argtypes = [ctypes.c_void_p, _D]
        L.och_set_rho.argtypes = [ctypes.c_void_p, _D]
        L.och_average_mass.restype = ctypes.c_double
        L.och_average_mass.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        L.och_average_free_energy.restype = ctypes.c_double
        L.och_average_free_energy.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        L.och_pressure_field.restype = ctypes.c_int
        L.och_pressure_field.argtypes = [ctypes.c_void_p, _D]
        L.och_average_pressure.restype = ctypes.c_double
        L.och_average_pressure.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        L.och_der_bulk_free_energy.argtypes = [ctypes.POINTER(abi.ModelParams), ctypes.c_int, _D, _D]
        L.och_set_mobility.argtypes = [ctypes.POINTER(abi.ModelParams), ctypes.c_int, _D, ctypes.c_double, _D]
        L.och_bulk_free_energy.restype = ctypes.c_double
        L.och_bulk_free_energy.argtypes = [ctypes.POINTER(abi.ModelParams), ctypes.c_int, _D, ctypes.c_int]
        L.och_init_density.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_void_p, _D]
        L.och_srand48.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.och_drand48.restype = ctypes.c_double
        L.och_drand48.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


class OracleSim:
    """One box of the CPU oracle (EulerCPU / EulerMobilityCPU / PseudospectralCPU)."""

    def __init__(self, params: abi.Params, rho: np.ndarray):
        self.params = params.copy()
        self.n = params.bins * params.n_species
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        assert rho.size == self.n
        self._h = lib().och_create(ctypes.byref(self.params), _ptr(rho))

    def step(self, n: int) -> None:
        lib().och_step(self._h, int(n))

    def rho(self) -> np.ndarray:
        out = np.empty(self.n)
        lib().och_get_rho(self._h, _ptr(out))
        return out

    def mobility(self) -> np.ndarray:
        out = np.empty(self.n)
        lib().och_get_mobility(self._h, _ptr(out))
        return out

    def set_rho(self, rho: np.ndarray) -> None:
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        lib().och_set_rho(self._h, _ptr(rho))

    def average_mass(self) -> tuple[float, bool]:
        nan = ctypes.c_int(0)
        v = lib().och_average_mass(self._h, ctypes.byref(nan))
        return v, bool(nan.value)

    def average_free_energy(self) -> tuple[float, bool]:
        nan = ctypes.c_int(0)
        v = lib().och_average_free_energy(self._h, ctypes.byref(nan))
        return v, bool(nan.value)

    def pressure(self) -> np.ndarray:
        """The pressure field (Landau only), layout of the density."""
        out = np.empty(self.n, dtype=np.float64)
        if lib().och_pressure_field(self._h, _ptr(out)) != 0:
            raise ValueError("this model does not support the pressure coupling")
        return out

    def average_pressure(self) -> float:
        bad = ctypes.c_int(0)
        v = lib().och_average_pressure(self._h, ctypes.byref(bad))
        if bad.value:
            raise ValueError("this model does not support the pressure coupling")
        return v

    def close(self) -> None:
        if self._h:
            lib().och_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def der_bulk_free_energy(model: abi.ModelParams, rho: np.ndarray, bins: int) -> np.ndarray:
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    out = np.zeros_like(rho)
    lib().och_der_bulk_free_energy(ctypes.byref(model), bins, _ptr(rho), _ptr(out))
    return out


def set_mobility(model: abi.ModelParams, rho: np.ndarray, M0: float) -> np.ndarray:
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    out = np.zeros_like(rho)
    lib().och_set_mobility(ctypes.byref(model), rho.size, _ptr(rho), M0, _ptr(out))
    return out


def init_density(dims, N, densities, initial_A=1e-2, initial_N_peaks=0, user_to_internal=1.0, seed=0):
    S = len(densities)
    out = np.empty(S * N ** dims)
    dens = np.ascontiguousarray(densities, dtype=np.float64)
    state = ctypes.c_uint64(0)
    lib().och_srand48(ctypes.byref(state), int(seed))
    lib().och_init_density(dims, N, S, _ptr(dens), initial_A, initial_N_peaks, user_to_internal,
                           ctypes.byref(state), _ptr(out))
    return out


def run_reference(dims: int, config_text: str, steps: int, workdir: Path) -> dict:
    """Run the reference's own integrators (oracle/_ref/ref_harness_<dims>D)
    on a TOML text; returns init/final rho, mobility, observables, seconds."""
    exe = REF_DIR / f"ref_harness_{dims}D"
    if not exe.exists():
        raise FileNotFoundError(exe)
    workdir = Path(workdir).resolve()
    workdir.mkdir(parents=True, exist_ok=True)
    cfg = workdir / "config.toml"
    cfg.write_text(config_text)
    prefix = workdir / "out"
    r = subprocess.run([str(exe), str(cfg), str(steps), str(prefix)], cwd=workdir, capture_output=True,
                       text=True, check=True)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("evolve_seconds")][-1]
    secs = float(line.split()[1])
    obs = np.loadtxt(str(prefix) + "_obs.txt")
    out = {
        "init": np.fromfile(str(prefix) + "_init.bin", dtype=np.float64),
        "final": np.fromfile(str(prefix) + "_final.bin", dtype=np.float64),
        "mobility": np.fromfile(str(prefix) + "_mobility.bin", dtype=np.float64),
        "obs_init": obs[0], "obs_final": obs[1], "seconds": secs,
    }
    ptxt = Path(str(prefix) + "_pressure.txt")
    if ptxt.exists():                       # Landau: the reference's pressure() and average_pressure()
        out["average_pressure"] = np.loadtxt(str(ptxt)).reshape(-1)
        out["pressure"] = np.fromfile(str(prefix) + "_pressure.bin", dtype=np.float64)
    return out


def rfftn(a: np.ndarray) -> np.ndarray:
    """Oracle forward real FFT (FFTW r2c semantics) of one real array."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    n = (ctypes.c_int * a.ndim)(*a.shape)
    hshape = a.shape[:-1] + (a.shape[-1] // 2 + 1,)
    out = np.empty(hshape + (2,))
    L = lib()
    L.och_rfftn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, _D, ctypes.c_size_t, _D,
                            ctypes.c_size_t]
    L.och_rfftn(a.ndim, n, 1, _ptr(a), a.size, out.ctypes.data_as(_D), int(np.prod(hshape)))
    return out[..., 0] + 1j * out[..., 1]


def irfftn(h: np.ndarray, shape) -> np.ndarray:
    """Oracle unnormalised inverse (FFTW c2r semantics)."""
    hh = np.ascontiguousarray(np.stack([h.real, h.imag], axis=-1), dtype=np.float64)
    n = (ctypes.c_int * len(shape))(*shape)
    out = np.empty(shape)
    L = lib()
    L.och_irfftn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, _D, ctypes.c_size_t, _D,
                             ctypes.c_size_t]
    L.och_irfftn(len(shape), n, 1, hh.ctypes.data_as(_D), int(np.prod(h.shape)), _ptr(out), out.size)
    return out


def radial_average_sq(field2d: np.ndarray, dx: float = 1.0) -> tuple[np.ndarray, np.ndarray]:
    """Radially averaged S(q) of a square 2D field: a restatement of the
    reference's utils/sq_from_traj.py:72-103 (radial_average_Sq with
    subtract_mean): |fft2(phi - mean)|^2 / N_cells, shells rint(|k| / dq)."""
    L = field2d.shape[0]
    n = L * L
    phi = field2d - field2d.mean()
    sk = np.abs(np.fft.fft2(phi)) ** 2 / n
    k = 2.0 * np.pi * np.fft.fftfreq(L, d=dx)
    kx, ky = np.meshgrid(k, k, indexing="ij")
    kk = np.sqrt(kx ** 2 + ky ** 2)
    dq = 2.0 * np.pi / (L * dx)
    shell = np.rint(kk / dq).astype(np.int64).ravel()
    sums = np.bincount(shell, weights=sk.ravel(), minlength=shell.max() + 1)
    counts = np.bincount(shell, minlength=shell.max() + 1)
    sq = np.zeros_like(sums)
    m = counts > 0
    sq[m] = sums[m] / counts[m]
    return np.arange(shell.max() + 1) * dq, sq


def sq_loss_of_run(params, rho0: np.ndarray, steps: int, target: np.ndarray) -> float:
    """sum_q (S(q) - S*(q))^2 of the oracle trajectory (2D, species 0)."""
    sim = OracleSim(params, rho0)
    sim.step(steps)
    N = params.N
    _, sq = radial_average_sq(sim.rho()[: N * N].reshape(N, N), params.dx)
    sim.close()
    return float(np.sum((sq - target) ** 2))
