"""Python mirror of the reference's simulation object over the C ABI.

``CahnHilliard`` plays the part of the reference's
``CahnHilliard<dims>`` + CUDA ``Integrator<dims>`` pair
(src/CahnHilliard.cpp:278-319, src/CUDA/integrators/CUDAIntegrator.cu):
``evolve()`` advances the device state, ``sync()`` copies it back,
``average_mass()`` / ``average_free_energy()`` reduce on the device.  Where
the reference calls ``critical()`` and exits, this raises ``ChgbError``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi

_D = ctypes.POINTER(ctypes.c_double)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


class CahnHilliard:
    def __init__(self, params: abi.Params, rho: np.ndarray | None = None, lib=None):
        self.lib = lib or abi.load_library()
        self.params = params.copy()
        self.n = params.bins * params.n_species
        h = ctypes.c_void_p()
        abi.check(self.lib, self.lib.chgb_create(ctypes.byref(self.params), ctypes.byref(h)))
        self._h = h
        if rho is not None:
            self.upload(rho)

    # -- state -------------------------------------------------------------
    def upload(self, rho: np.ndarray, mobility: np.ndarray | None = None) -> None:
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        if rho.size != self.n:
            raise ValueError(f"expected {self.n} values, got {rho.size}")
        mob = None
        if mobility is not None:
            mob = np.ascontiguousarray(mobility, dtype=np.float64).reshape(-1)
            if mob.size != self.n:
                raise ValueError(f"expected {self.n} mobility values, got {mob.size}")
        abi.check(self.lib, self.lib.chgb_upload(self._h, _ptr(rho), _ptr(mob) if mob is not None else None),
                  self._h)

    def evolve(self, nsteps: int = 1) -> None:
        abi.check(self.lib, self.lib.chgb_step(self._h, int(nsteps)), self._h)

    def sync(self, with_mobility: bool = False):
        rho = np.empty(self.n)
        mob = np.empty(self.n) if with_mobility else None
        abi.check(self.lib, self.lib.chgb_download(self._h, _ptr(rho), _ptr(mob) if mob is not None else None),
                  self._h)
        return (rho, mob) if with_mobility else rho

    def rho(self) -> np.ndarray:
        return self.sync()

    def mobility(self) -> np.ndarray:
        return self.sync(with_mobility=True)[1]

    def synchronize(self) -> None:
        abi.check(self.lib, self.lib.chgb_synchronize(self._h), self._h)

    def device_rho(self) -> int:
        p = _D()
        abi.check(self.lib, self.lib.chgb_device_rho(self._h, ctypes.byref(p)), self._h)
        return ctypes.cast(p, ctypes.c_void_p).value

    def set_stream(self, stream_handle: int | None) -> None:
        abi.check(self.lib, self.lib.chgb_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)), self._h)

    @property
    def launches(self) -> int:
        return int(self.lib.chgb_launch_count(self._h))

    @property
    def kernel_variant(self) -> int:
        return int(self.lib.chgb_kernel_variant(self._h))

    def structure_factor(self, species: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """(q, S(q)) of a 2D box, utils/sq_from_traj.py:72-103 of the reference."""
        nb = int(self.lib.chgb_structure_factor_bins(self.params.N))
        sq = np.empty(nb)
        abi.check(self.lib, self.lib.chgb_structure_factor(self._h, species, _ptr(sq), nb), self._h)
        dq = 2.0 * np.pi / (self.params.N * self.params.dx)
        return np.arange(nb) * dq, sq

    # -- observables ---------------------------------------------------------
    def observables(self, raise_on_nan: bool = True) -> tuple[float, float, bool]:
        mass, fe, nan = ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
        code = self.lib.chgb_observables(self._h, ctypes.byref(mass), ctypes.byref(fe), ctypes.byref(nan))
        if code != abi.CHGB_ERR_NAN or raise_on_nan:
            abi.check(self.lib, code, self._h)
        return mass.value, fe.value, bool(nan.value)

    def average_mass(self) -> float:
        return self.observables()[0]

    def average_free_energy(self) -> float:
        return self.observables()[1]

    def pressure(self) -> np.ndarray:
        """The pressure field of the current state (Landau only), the
        reference's CahnHilliard::pressure(); same layout as the density."""
        out = np.empty(self.params.bins * self.params.n_species, dtype=np.float64)
        abi.check(self.lib, self.lib.chgb_pressure(self._h, out.ctypes.data_as(abi._D), None), self._h)
        return out

    def average_pressure(self) -> float:
        """The reference's average_pressure() (Landau only; no V_bin factor)."""
        v = ctypes.c_double()
        abi.check(self.lib, self.lib.chgb_pressure(self._h, None, ctypes.byref(v)), self._h)
        return v.value

    # -- lifetime ------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.chgb_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Adjoint:
    """Checkpointed forward pass and hand-written adjoint (chgb_adjoint_*)."""

    def __init__(self, params: abi.Params, nsteps: int, checkpoint_every: int = 0, lib=None):
        self.lib = lib or abi.load_library()
        self.params = params.copy()
        self.nsteps = int(nsteps)
        a = ctypes.c_void_p()
        abi.check(self.lib, self.lib.chgb_adjoint_create(ctypes.byref(self.params), self.nsteps,
                                                         int(checkpoint_every), ctypes.byref(a)))
        self._a = a
        self.n = params.bins
        self.nbins = int(self.lib.chgb_structure_factor_bins(params.N))

    def forward(self, rho0: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """Run the trajectory; returns (S(q) of the final state, final field)."""
        rho0 = np.ascontiguousarray(rho0, dtype=np.float64).reshape(-1)
        sq = np.empty(self.nbins)
        rho_t = np.empty(self.n)
        abi.check(self.lib, self.lib.chgb_adjoint_forward(self._a, _ptr(rho0), _ptr(sq), _ptr(rho_t)))
        return sq, rho_t

    def backward(self, dl_dsq: np.ndarray | None = None, dl_drho_t: np.ndarray | None = None):
        """Returns (dL/drho0, [dL/deps, dL/dk, dL/dM])."""
        g0 = np.empty(self.n)
        g3 = np.empty(3)
        a = None if dl_dsq is None else np.ascontiguousarray(dl_dsq, dtype=np.float64)
        b = None if dl_drho_t is None else np.ascontiguousarray(dl_drho_t, dtype=np.float64).reshape(-1)
        abi.check(self.lib, self.lib.chgb_adjoint_backward(self._a, _ptr(a) if a is not None else None,
                                                           _ptr(b) if b is not None else None, _ptr(g0), _ptr(g3)))
        return g0, g3

    @property
    def launches(self) -> int:
        return int(self.lib.chgb_adjoint_launch_count(self._a))

    def close(self) -> None:
        if getattr(self, "_a", None):
            self.lib.chgb_adjoint_destroy(self._a)
            self._a = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent boxes stepped together (chgb_batch_*).  Each replica
    has its own parameters; replica i is addressed by its index."""

    def __init__(self, params_list, lib=None):
        self.lib = lib or abi.load_library()
        self.params = [p.copy() for p in params_list]
        arr = (abi.Params * len(self.params))(*self.params)
        b = ctypes.c_void_p()
        abi.check(self.lib, self.lib.chgb_batch_create(arr, len(self.params), ctypes.byref(b)))
        self._b = b

    def __len__(self):
        return len(self.params)

    def _n(self, i):
        return self.params[i].bins * self.params[i].n_species

    def upload(self, i: int, rho: np.ndarray) -> None:
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        if rho.size != self._n(i):
            raise ValueError("wrong field size")
        abi.check(self.lib, self.lib.chgb_batch_upload(self._b, i, _ptr(rho)))

    def step(self, nsteps: int) -> None:
        abi.check(self.lib, self.lib.chgb_batch_step(self._b, int(nsteps)))

    def synchronize(self) -> None:
        abi.check(self.lib, self.lib.chgb_batch_synchronize(self._b))

    def download(self, i: int) -> np.ndarray:
        out = np.empty(self._n(i))
        abi.check(self.lib, self.lib.chgb_batch_download(self._b, i, _ptr(out)))
        return out

    def observables(self, i: int) -> tuple[float, float, bool]:
        h = self.lib.chgb_batch_replica(self._b, i)
        mass, fe, nan = ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
        code = self.lib.chgb_observables(h, ctypes.byref(mass), ctypes.byref(fe), ctypes.byref(nan))
        if code not in (abi.CHGB_OK, abi.CHGB_ERR_NAN):
            abi.check(self.lib, code, h)
        return mass.value, fe.value, bool(nan.value)

    @property
    def launches(self) -> int:
        return int(self.lib.chgb_batch_launch_count(self._b))

    @property
    def euler_tile(self) -> int:
        return int(self.lib.chgb_batch_euler_tile(self._b))

    def close(self) -> None:
        if getattr(self, "_b", None):
            self.lib.chgb_batch_destroy(self._b)
            self._b = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def der_bulk_free_energy(model: abi.ModelParams, d_rho: int, d_out: int, bins: int, stream: int = 0, lib=None):
    """Device hook: d_out = f'(d_rho) for `bins` cells (device pointers as ints)."""
    lib = lib or abi.load_library()
    abi.check(lib, lib.chgb_der_bulk_free_energy(ctypes.byref(model), ctypes.c_void_p(d_rho),
                                                 ctypes.c_void_p(d_out), int(bins), ctypes.c_void_p(stream)))


def set_mobility(model: abi.ModelParams, d_rho: int, M0: float, d_out: int, n: int, stream: int = 0, lib=None):
    lib = lib or abi.load_library()
    abi.check(lib, lib.chgb_set_mobility(ctypes.byref(model), ctypes.c_void_p(d_rho), float(M0),
                                         ctypes.c_void_p(d_out), int(n), ctypes.c_void_p(stream)))
