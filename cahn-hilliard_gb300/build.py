"""Build libchgb.so (sm_103a) in-tree with nvcc, plus the host driver binaries.

    python cahn-hilliard_gb300/build.py

Each CUDA translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
cahn-hilliard_gb300/lib/libchgb.so.  Objects are rebuilt only when a source
or header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
BUILD = PKG / "_build"
LIB = PKG / "lib"
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no implicit a*b+c contraction.  Every FMA of the hot kernels is
# an explicit fma(); without implicit contraction the same expression rounds
# the same way in every kernel that inlines it (single box, split, batched),
# which keeps those paths bit-identical, and matches the oracle's
# -ffp-contract=off arithmetic for the model formulas.  Host code (the tables
# built at create, the drivers) takes -ffp-contract=off too: GCC contracts by
# default on aarch64 but not on x86-64, and the tables must not depend on the
# machine.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
              "-fmad=false"]
CUDA_SOURCES = ["api.cu", "euler.cu", "fields.cu", "spectral.cu", "psmob.cu", "psmob_gmres.cu", "batch.cu", "sq.cu",
                "adjoint.cu",
                "noalloc.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


def _newest_header() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max(p.stat().st_mtime for p in hs)


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")


def build_library(force: bool = False, extra: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    extra = extra or []
    hdr = _newest_header()
    jobs = []
    for name in CUDA_SOURCES:
        src = CSRC / name
        obj = BUILD / (src.stem + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr):
            jobs.append((src, obj))
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(lambda a: _compile(a[0], a[1], extra), jobs))
    out = LIB / "libchgb.so"
    objs = [str(BUILD / (Path(n).stem + ".o")) for n in CUDA_SOURCES]
    if force or jobs or not out.exists():
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(out), *objs, "-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return out


BOUNDS_CHECKED = ["euler.cu", "spectral.cu"]   # the translation units whose kernels carry CHGB_BC checks


def build_bounds_check_library(force: bool = False) -> Path:
    """lib/libchgb_bc.so: libchgb with the explicit kernels' index checks
    compiled in (-DCHGB_BOUNDS_CHECK; read them with chgb_bounds_report).  The
    other translation units are the normal build's objects.  Not part of
    build(): the test that uses it builds it."""
    build_library()
    hdr = _newest_header()
    objs = []
    jobs = []
    for name in CUDA_SOURCES:
        src = CSRC / name
        if name in BOUNDS_CHECKED:
            obj = BUILD / (src.stem + "_bc.o")
            if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr):
                jobs.append((src, obj))
        else:
            obj = BUILD / (src.stem + ".o")
        objs.append(str(obj))
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(lambda a: _compile(a[0], a[1], ["-DCHGB_BOUNDS_CHECK"]), jobs))
    out = LIB / "libchgb_bc.so"
    if force or jobs or not out.exists() or out.stat().st_mtime < (LIB / "libchgb.so").stat().st_mtime:
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", str(out), *objs, "-lcudart", "-ldl"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return out


def build_host(force: bool = False) -> list[Path]:
    """The C++ drop-in drivers ch_{1,2,3}D (host/), linked against libchgb.so."""
    srcs = sorted(HOST.glob("*.cpp"))
    if not srcs:
        return []
    BUILD.mkdir(exist_ok=True)
    outs = []
    lib = LIB / "libchgb.so"
    newest = max([p.stat().st_mtime for p in srcs + list(HOST.glob("*.h"))] + [lib.stat().st_mtime])
    cxx = shutil.which("g++") or "g++"
    cuda_inc = Path(nvcc()).resolve().parent.parent / "include"

    def one(d: int) -> Path:
        exe = LIB / f"ch_{d}D"
        if force or not exe.exists() or exe.stat().st_mtime < newest:
            cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", f"-DDIM={d}", f"-I{INCLUDE}", f"-I{cuda_inc}",
                   *map(str, srcs),
                   f"-L{LIB}", "-lchgb", f"-Wl,-rpath,{LIB}", "-o", str(exe)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"host build failed:\n{r.stdout}\n{r.stderr}")
        return exe

    with ThreadPoolExecutor(max_workers=3) as ex:
        outs = list(ex.map(one, (1, 2, 3)))
    return outs


def build_probe(force: bool = False) -> Path:
    """lib/chgb_fp64_peak: the FP64 instruction-rate probe bench.py reports against."""
    src = CSRC / "fp64_peak.cu"
    exe = LIB / "chgb_fp64_peak"
    if force or not exe.exists() or exe.stat().st_mtime < src.stat().st_mtime:
        LIB.mkdir(exist_ok=True)
        r = subprocess.run([nvcc(), *ARCH, "-O3", "-o", str(exe), str(src)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"probe build failed:\n{r.stdout}\n{r.stderr}")
    return exe


def build(force: bool = False) -> None:
    build_library(force)
    with ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_host, force)
        b = ex.submit(build_probe, force)
        a.result()
        b.result()


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built", LIB / "libchgb.so")
