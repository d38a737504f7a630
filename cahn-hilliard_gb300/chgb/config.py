"""TOML configuration -> C-ABI parameters, following the reference's constructors.

The reference reads its TOML keys in the constructors of its objects; this
module applies the same keys, defaults, unit rescalings and rejections:

* ``CahnHilliard`` (src/CahnHilliard.cpp:34-163): ``N`` (power of two), ``k``,
  ``dt``, ``dx``, ``distance_scaling_factor``, ``integrator``,
  ``initial_density`` / ``initial_A`` / ``initial_N_peaks``; dx *= u,
  k *= u^5, rho /= u^3 with u = 1/distance_scaling_factor.
* models (src/models/Landau.cpp:16-36, SimpleWertheim.cpp:20-34,
  SalehWertheim.cpp:19-41) and ``Delta`` (src/utils/Delta.cpp:15-42).
* mobility (src/mobility/IMobility.cpp:18-57, ConstantMobility.h:18-22,
  FreeEnergyMobility.h:18-22): M /= u.
* pseudospectral (src/integrators/PseudospectralCPU.cpp:24-25): S *= u^3.
* ``Integrator::validate`` (src/integrators/Integrator.cpp:38-42).

Errors the reference reports with ``critical()`` (log + exit(1)) raise
``ConfigError`` here.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi


class ConfigError(ValueError):
    pass


def _get(cfg: dict, path: str, default=None, mandatory: bool = False):
    node = cfg
    for part in path.split("."):
        if not isinstance(node, dict) or part not in node:
            if mandatory:
                raise ConfigError(f"Mandatory option '{path}' not found")
            return default
        node = node[part]
    return node


def _as_int(v, path):
    if isinstance(v, bool):
        raise ConfigError(f"Option '{path}' is not an integer")
    if isinstance(v, int):
        return v
    if isinstance(v, float) and v.is_integer():
        return int(v)
    raise ConfigError(f"Option '{path}' is not an integer")


def _as_float(v, path):
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise ConfigError(f"Option '{path}' is not a number")
    return float(v)


def _array_values(cfg, path, size, kind=float):
    """Object::_config_array_values (src/Object.h:32-78): a scalar of the exact
    TOML type broadcasts to `size` entries; otherwise an array of that size."""
    v = _get(cfg, path, mandatory=True)
    want = (float,) if kind is float else (int,)
    if isinstance(v, want) and not isinstance(v, bool):
        return [kind(v)] * size
    if isinstance(v, list):
        if not all(isinstance(e, want) and not isinstance(e, bool) for e in v):
            raise ConfigError(f"Option '{path}': cannot convert element")
        out = [kind(e) for e in v]
        if len(out) != size:
            raise ConfigError(f"Option '{path}' should be a single value or an array of size {size}, not {len(out)}")
        return out
    raise ConfigError(f"Option '{path}' should be a single value or an array of size {size}, not 0")


def delta_value(node, path: str) -> float:
    """Wertheim bonding volume Delta from a number or a {T, deltaH, deltaS,
    salt, sticky_size} table (src/utils/Delta.cpp:15-42)."""
    if isinstance(node, (int, float)) and not isinstance(node, bool):
        return float(node)
    if isinstance(node, dict):
        d = float(node.get("value", 0.0))
        if d == 0.0:
            for key in ("T", "deltaH", "deltaS"):
                if key not in node:
                    raise ConfigError(f"Mandatory option '{key}' not found")
            T = float(node["T"])
            salt = float(node.get("salt", 1.0))
            L_DNA = int(node.get("sticky_size", 6))
            dH = float(node["deltaH"])
            dS = float(node["deltaS"])
            dS_salt = 0.368 * (L_DNA - 1.0) * math.log(salt)
            dG = dH - T * (dS + dS_salt)
            k_B = 1.9872036
            d = 1.6606 * math.exp(-dG / (k_B * T))
        return d
    raise ConfigError(f"A delta must be specified either as a single number or as a table of values ({path})")


@dataclass
class Setup:
    params: abi.Params
    steps: int = 0
    seed: int = 0
    print_every: int = 0
    user_to_internal: float = 1.0
    initial_density: list = field(default_factory=list)
    initial_A: float = 1e-2
    initial_N_peaks: int = 0
    load_from: str | None = None
    model_name: str = "landau"
    integrator_name: str = "euler"
    use_CUDA: bool = False


def model_params(cfg: dict, user_to_internal: float) -> tuple[str, abi.ModelParams]:
    name = _get(cfg, "free_energy", mandatory=True)
    if name not in abi.MODELS:
        raise ConfigError(f"Unsupported free energy model '{name}'")
    u = user_to_internal
    m = abi.ModelParams()
    m.kind = abi.MODELS[name]
    m.n_species = abi.N_SPECIES[name]
    m.density_conversion_factor = u ** 3
    if name == "landau":
        if _get(cfg, "landau.epsilon") is not None:
            m.epsilon = _as_float(_get(cfg, "landau.epsilon"), "landau.epsilon")
        elif _get(cfg, "landau.T") is not None:
            m.epsilon = 1 - _as_float(_get(cfg, "landau.T"), "landau.T")
        else:
            raise ConfigError("The Landau free energy requires either 'epsilon' or 'T' to be set")
        if u != 1.0:
            raise ConfigError("The Landau free energy does not support distance_scaling_factor values different from 1.0")
    elif name == "simple_wertheim":
        m.valence = _as_int(_get(cfg, "wertheim.valence", mandatory=True), "wertheim.valence")
        B2 = _as_float(_get(cfg, "wertheim.B2", mandatory=True), "wertheim.B2")
        reg = _as_float(_get(cfg, "wertheim.regularisation_delta", 0.0), "wertheim.regularisation_delta")
        delta = delta_value(_get(cfg, "wertheim.delta", mandatory=True), "wertheim.delta")
        m.B2 = B2 * u ** 3
        m.delta = delta * u ** 3
        m.regularisation_delta = reg / u ** 3
    else:
        m.B2 = _as_float(_get(cfg, "saleh.B2", mandatory=True), "saleh.B2") * u ** 3
        m.B3 = _as_float(_get(cfg, "saleh.B3", 0.0), "saleh.B3") * (u ** 3) ** 2
        m.delta_AA = delta_value(_get(cfg, "saleh.delta_AA", mandatory=True), "saleh.delta_AA") * u ** 3
        m.delta_BB = delta_value(_get(cfg, "saleh.delta_BB", mandatory=True), "saleh.delta_BB") * u ** 3
        val = _array_values(cfg, "saleh.valence", 3, int)
        for i in range(3):
            m.saleh_valence[i] = val[i]
    return name, m


def setup_from_config(cfg: dict) -> Setup:
    """Build the parameters of one box from a parsed TOML table."""
    internal_to_user = _as_float(_get(cfg, "distance_scaling_factor", 1.0), "distance_scaling_factor")
    u = 1.0 / internal_to_user
    name, m = model_params(cfg, u)
    S = int(m.n_species)
    p = abi.Params()
    p.model = m
    N = _as_int(_get(cfg, "N", mandatory=True), "N")
    if N <= 0 or (N & (N - 1)) != 0:
        raise ConfigError("N should be a power of 2")
    p.N = N
    p.dt = _as_float(_get(cfg, "dt", mandatory=True), "dt")
    p.dx = _as_float(_get(cfg, "dx", 1.0), "dx") * u
    ks = _array_values(cfg, "k", S, float)
    for i in range(S):
        p.k[i] = ks[i] * u ** 5
    integ = _get(cfg, "integrator", "euler")
    if integ not in abi.INTEGRATORS:
        raise ConfigError(f"Unsupported integrator {integ}")
    p.integrator = abi.INTEGRATORS[integ]
    if integ == "pseudospectral_mobility":
        # src/integrators/PseudospectralMobilityCPU.cpp:204-208
        p.use_gmres = 1 if _get(cfg, "pseudospectral.use_gmres", False) else 0
        p.gmres_restart = _as_int(_get(cfg, "pseudospectral.gmres_restart", 30), "pseudospectral.gmres_restart")
        p.gmres_max_iter = _as_int(_get(cfg, "pseudospectral.gmres_max_iter", 200), "pseudospectral.gmres_max_iter")
        p.gmres_tol = _as_float(_get(cfg, "pseudospectral.gmres_tol", 1e-10), "pseudospectral.gmres_tol")
    mob = _get(cfg, "mobility.type", "constant")
    if mob not in abi.MOBILITIES:
        raise ConfigError(f"Unknown mobility type: {mob}")
    p.mobility_type = abi.MOBILITIES[mob]
    p.M = _as_float(_get(cfg, "mobility.M", 1.0), "mobility.M") / u
    if mob == "regularised":
        # src/mobility/IMobility.cpp:48-55, RegularisedMobility.h:19-22
        rho_min = _get(cfg, "mobility.rho_min")
        if rho_min is None:
            raise ConfigError("For 'regularised' mobility, 'rho_min' must be specified")
        p.rho_min = _as_float(rho_min, "mobility.rho_min") / u
    elif mob == "gel":
        # src/mobility/IMobility.cpp:30-47, GelMobility.h:19-25
        keys = ("mobility.phi_critical", "mobility.c_0", "mobility.M_c", "landau.epsilon")
        vals = [_get(cfg, k_) for k_ in keys]
        if any(v is None for v in vals):
            raise ConfigError("For 'gel' mobility, 'phi_critical', 'c_0', 'M_c', and 'landau.epsilon' must be "
                              "specified")
        phi_c, c0, M_c, eps = (_as_float(v, k_) for v, k_ in zip(vals, keys))
        p.gel_phi_critical = phi_c
        p.gel_c0 = c0
        p.gel_M_c = M_c / u
        p.gel_beta_delta_F = 10.0 / (1.0 - eps) - math.log(24000.0)
    p.splitting_S = _as_float(_get(cfg, "pseudospectral.S", 0.0), "pseudospectral.S")
    if integ != "pseudospectral_mobility":
        # src/integrators/PseudospectralCPU.cpp:24 scales S; PseudospectralMobilityCPU.cpp:22 does not
        p.splitting_S *= u ** 3
    p.use_dealias = 1 if _get(cfg, "pseudospectral.use_dealias", False) else 0
    if mob != "constant" and integ not in ("euler_mobility", "pseudospectral_mobility"):
        raise ConfigError("The selected integrator only supports constant mobility")
    if mob == "free_energy" and name != "simple_wertheim":
        raise ConfigError("this model does not support mobility coupling")
    st = Setup(params=p, user_to_internal=u, model_name=name, integrator_name=integ)
    st.steps = _as_int(_get(cfg, "steps", mandatory=True), "steps")
    if st.steps < 0:
        raise ConfigError("steps should be a number larger than 0")
    st.seed = _as_int(_get(cfg, "seed", 0), "seed")
    st.print_every = _as_int(_get(cfg, "print_every", 0), "print_every")
    st.use_CUDA = bool(_get(cfg, "use_CUDA", False))
    st.load_from = _get(cfg, "load_from")
    if st.load_from is None:
        if _get(cfg, "initial_density") is None:
            raise ConfigError("Either 'initial_density' or 'load_from' should be specified")
        st.initial_density = _array_values(cfg, "initial_density", S, float)
        st.initial_A = _as_float(_get(cfg, "initial_A", 1e-2), "initial_A")
        st.initial_N_peaks = _as_int(_get(cfg, "initial_N_peaks", 0), "initial_N_peaks")
    return st


def params(dims: int, N: int, integrator: str = "euler", model: str = "landau", *, dt: float, dx: float = 1.0,
           k=1.0, M: float = 1.0, mobility: str = "constant", S: float = 0.0, use_dealias: bool = False,
           **model_kw) -> abi.Params:
    """Direct constructor of the C-ABI parameters (internal units)."""
    p = abi.Params()
    p.dims, p.N = dims, N
    p.integrator = abi.INTEGRATORS[integrator]
    p.mobility_type = abi.MOBILITIES[mobility]
    p.dt, p.dx, p.M = dt, dx, M
    p.splitting_S = S
    p.use_dealias = int(bool(use_dealias))
    m = abi.ModelParams()
    m.kind = abi.MODELS[model]
    m.n_species = abi.N_SPECIES[model]
    m.density_conversion_factor = model_kw.pop("density_conversion_factor", 1.0)
    sv = model_kw.pop("saleh_valence", (4, 4, 4))
    for i in range(3):
        m.saleh_valence[i] = int(sv[i])
    for key, v in model_kw.items():
        setattr(m, key, v)
    p.model = m
    ks = list(k) if isinstance(k, (list, tuple)) else [k] * m.n_species
    for i, kv in enumerate(ks):
        p.k[i] = kv
    return p


# ---------------------------------------------------------------------------
# initial density: src/CahnHilliard.cpp:133-161 with the POSIX drand48 stream
# seeded as in src/main.cpp:36
# ---------------------------------------------------------------------------
_A48 = 0x5DEECE66D
_C48 = 0xB
_MASK48 = (1 << 48) - 1


def drand48_stream(seed: int, count: int) -> np.ndarray:
    """The first `count` values of drand48() after srand48(seed), vectorised
    with the affine jump X_{n+B} = A_B X_n + C_B (mod 2^48)."""
    x0 = ((seed & 0xFFFFFFFF) << 16) | 0x330E
    out = np.empty(count, dtype=np.uint64)
    B = min(count, 4096)
    x = x0
    for i in range(B):
        x = (_A48 * x + _C48) & _MASK48
        out[i] = x
    # affine map of B steps
    aB, cB = 1, 0
    for _ in range(B):
        aB, cB = (_A48 * aB) & _MASK48, (_A48 * cB + _C48) & _MASK48
    aB64, cB64 = np.uint64(aB), np.uint64(cB)
    mask = np.uint64(_MASK48)
    pos = B
    while pos < count:
        n = min(B, count - pos)
        prev = out[pos - B:pos - B + n]
        with np.errstate(over="ignore"):
            out[pos:pos + n] = (prev * aB64 + cB64) & mask
        pos += n
    return np.ldexp(out.astype(np.float64), -48)


def init_density(dims: int, N: int, densities, initial_A: float = 1e-2, initial_N_peaks: int = 0,
                 user_to_internal: float = 1.0, seed: int = 0) -> np.ndarray:
    """Species-major FP64 density of src/CahnHilliard.cpp:133-161."""
    S = len(densities)
    bins = N ** dims
    r = drand48_stream(seed, bins * S).reshape(bins, S)
    initial_k = 2 * math.pi * initial_N_peaks / float(N)
    modulation = initial_A * np.cos(initial_k * np.arange(bins, dtype=np.float64))
    if initial_N_peaks == 0:
        rf = r - 0.5
    else:
        rf = 1.0 + 0.02 * (r - 0.5)
    rho = np.empty((S, bins))
    for i, avg in enumerate(densities):
        if avg != 0.0:
            rho[i] = avg * (1.0 + 2.0 * modulation * rf[:, i])
        else:
            rho[i] = 2.0 * modulation * rf[:, i]
    rho /= user_to_internal ** 3
    return rho.reshape(-1)
