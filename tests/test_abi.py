"""CPU tests of the C-ABI library: it loads, exports every declared symbol,
its structs match the C layout, and it rejects what the reference rejects --
all without a GPU (validation happens before any CUDA call)."""
import ctypes
import subprocess
import textwrap

import pytest

from chgb import abi, config


@pytest.fixture(scope="module")
def lib():
    return abi.load_library()


def test_library_exports_every_declared_symbol(lib):
    declared = abi.declared_symbols()
    assert len(declared) >= 14
    for name in declared:
        assert hasattr(lib, name), name
        assert name in abi.SIGNATURES, name


def test_bounds_check_library_builds_and_exports_every_declared_symbol():
    """libchgb_bc.so (the bounds-check build: euler.cu and spectral.cu with
    -DCHGB_BOUNDS_CHECK) compiles here and exports what the header declares;
    the GPU test runs it."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(abi.__file__).resolve().parent.parent))
    import build
    bc = abi.load_library(build.build_bounds_check_library())
    for name in abi.declared_symbols():
        assert hasattr(bc, name), name


def test_abi_version(lib):
    assert lib.chgb_abi_version() == abi.CHGB_ABI_VERSION


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(textwrap.dedent(f"""
        #include <stdio.h>
        #include <stddef.h>
        #include "{abi.HEADER_PATH}"
        int main(void) {{
            printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(chgb_params), sizeof(chgb_model_params),
                   offsetof(chgb_params, model), offsetof(chgb_params, splitting_S),
                   offsetof(chgb_model_params, B2), offsetof(chgb_model_params, density_conversion_factor),
                   offsetof(chgb_params, rho_min), offsetof(chgb_params, gel_beta_delta_F),
                   offsetof(chgb_params, gmres_tol));
            return 0;
        }}"""))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    got = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    want = [ctypes.sizeof(abi.Params), ctypes.sizeof(abi.ModelParams), abi.Params.model.offset,
            abi.Params.splitting_S.offset, abi.ModelParams.B2.offset,
            abi.ModelParams.density_conversion_factor.offset, abi.Params.rho_min.offset,
            abi.Params.gel_beta_delta_F.offset, abi.Params.gmres_tol.offset]
    assert got == want


def _create(lib, p):
    h = ctypes.c_void_p()
    code = lib.chgb_create(ctypes.byref(p), ctypes.byref(h))
    return code, h


@pytest.mark.parametrize("mutate,code,msg", [
    (lambda p: setattr(p, "N", 48), abi.CHGB_ERR_INVALID, "power of 2"),
    (lambda p: setattr(p, "N", 2), abi.CHGB_ERR_INVALID, "power of 2"),
    (lambda p: setattr(p, "dims", 4), abi.CHGB_ERR_INVALID, "dims"),
    (lambda p: setattr(p, "mobility_type", abi.MOBILITIES["free_energy"]), abi.CHGB_ERR_UNSUPPORTED,
     "only supports constant mobility"),
    (lambda p: setattr(p, "integrator", 7), abi.CHGB_ERR_INVALID, "integrator"),
    (lambda p: setattr(p, "mobility_type", abi.MOBILITIES["gel"]), abi.CHGB_ERR_INVALID, "c_0"),
    (lambda p: (setattr(p, "mobility_type", abi.MOBILITIES["regularised"]),
                setattr(p, "integrator", abi.INTEGRATORS["pseudospectral"])), abi.CHGB_ERR_UNSUPPORTED,
     "only supports constant mobility"),
    (lambda p: setattr(p, "mobility_type", 9), abi.CHGB_ERR_INVALID, "mobility type"),
    (lambda p: setattr(p, "kernel_variant", 6), abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: (setattr(p, "kernel_variant", 5), setattr(p, "integrator", abi.INTEGRATORS["euler_mobility"])),
     abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: (setattr(p, "kernel_variant", 5), setattr(p, "integrator", abi.INTEGRATORS["pseudospectral"])),
     abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: (setattr(p, "kernel_variant", 5), setattr(p, "dims", 1)), abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: (setattr(p, "kernel_variant", 5), setattr(p, "N", 16)), abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: (setattr(p, "kernel_variant", 5), setattr(p.model, "kind", abi.MODELS["simple_wertheim"])),
     abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: (setattr(p, "kernel_variant", 4), setattr(p, "N", 128)), abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: (setattr(p, "kernel_variant", 4), setattr(p, "integrator", abi.INTEGRATORS["euler_mobility"])),
     abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: (setattr(p, "kernel_variant", 3), setattr(p, "N", 1024)), abi.CHGB_ERR_INVALID, "kernel_variant"),
    (lambda p: setattr(p, "dt", -1.0), abi.CHGB_ERR_INVALID, "positive"),
])
def test_create_rejects_invalid_parameters(lib, mutate, code, msg):
    p = config.params(2, 64, "euler", "landau", dt=0.01, epsilon=0.9)
    mutate(p)
    got, h = _create(lib, p)
    assert got == code
    assert h.value is None
    assert msg in lib.chgb_last_error(None).decode()


@pytest.mark.parametrize("integrator,N,variant", [("euler", 1024, 3), ("pseudospectral", 64, 3), ("euler", 128, 4),
                                                 ("euler", 64, 5)])
def test_adjoint_rejects_kernel_variants_where_unsupported(lib, integrator, N, variant):
    p = config.params(2, N, integrator, "landau", dt=0.01, epsilon=0.9)
    p.kernel_variant = variant
    a = ctypes.c_void_p()
    assert lib.chgb_adjoint_create(ctypes.byref(p), 10, 0, ctypes.byref(a)) == abi.CHGB_ERR_INVALID
    assert a.value is None
    assert "kernel_variant" in lib.chgb_last_error(None).decode()


def test_free_energy_mobility_needs_simple_wertheim(lib):
    p = config.params(2, 64, "euler_mobility", "landau", dt=0.01, mobility="free_energy", epsilon=0.9)
    got, _ = _create(lib, p)
    assert got == abi.CHGB_ERR_UNSUPPORTED
    assert "mobility coupling" in lib.chgb_last_error(None).decode()


def test_hooks_validate_arguments(lib):
    m = abi.ModelParams()
    m.kind = abi.MODELS["landau"]
    m.n_species = 1
    assert lib.chgb_der_bulk_free_energy(ctypes.byref(m), None, None, 4, None) == abi.CHGB_ERR_INVALID
    x = ctypes.c_void_p(16)
    assert lib.chgb_set_mobility(ctypes.byref(m), x, 1.0, x, 4, None) == abi.CHGB_ERR_UNSUPPORTED
    assert lib.chgb_step(None, 1) == abi.CHGB_ERR_INVALID
    assert lib.chgb_destroy(None) == abi.CHGB_OK


def test_bounds_report_needs_the_bounds_check_build(lib):
    """The normal build answers chgb_bounds_report with CHGB_ERR_UNSUPPORTED
    (and a cleared record) without touching the device."""
    first = ctypes.c_ulonglong(7)
    assert lib.chgb_bounds_report(ctypes.byref(first)) == abi.CHGB_ERR_UNSUPPORTED
    assert first.value == 0
    assert "bounds-check build" in lib.chgb_last_error(None).decode()
    assert lib.chgb_bounds_report(None) == abi.CHGB_ERR_INVALID
