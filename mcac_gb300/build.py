"""Builds the native parts of the package in-tree.

* ``mcac_gb300/_build/libmcacg.so`` -- the product: CUDA kernels for sm_103a
  and the C++ host layer behind include/mcacg.h.
* ``oracle/_build/libmcac_oracle.so`` -- the CPU restatement of the reference
  algorithm (test infrastructure, never loaded by the product).
* ``oracle/_ref/`` -- the reference itself, built from its sources by
  oracle/ref.mk, only where the reference sources are present.

Floating-point contraction is disabled everywhere (``-fmad=false`` for device
code, ``-ffp-contract=off`` for host code) because the exact FP64 paths
reproduce the reference's rounding operation by operation.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "mcac_gb300"
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"
LIB = BUILD / "libmcacg.so"
ORACLE_LIB = ORACLE_BUILD / "libmcac_oracle.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", f"-I{ROOT / 'include'}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
             f"-I{CUDA_HOME / 'include'}", f"-I{ROOT / 'include'}"]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_library(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.hpp")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "mcacg.h"]
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([NVCC] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if jobs or not LIB.exists():
        tmp = BUILD / "libmcacg.so.tmp"
        _run([NVCC] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] +
             ["-cudart", "static", "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    srcs = sorted(ORACLE.glob("*.c"))
    hdrs = sorted(ORACLE.glob("*.h"))
    if srcs and _stale(ORACLE_LIB, srcs + hdrs):
        tmp = ORACLE_BUILD / "libmcac_oracle.so.tmp"
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
              "-o", str(tmp)] + [str(s) for s in srcs] + ["-lm"])
        os.replace(tmp, ORACLE_LIB)
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def reference_dir() -> Path:
    """The reference's source directory, from the MCAC_REFERENCE environment
    variable (the golden-vector generators need it; there is no default)."""
    ref = os.environ.get("MCAC_REFERENCE")
    if not ref or not (Path(ref) / "src" / "calcul.cpp").exists():
        raise RuntimeError("set MCAC_REFERENCE to the reference's source directory (the one holding src/calcul.cpp)")
    return Path(ref)


def build_reference(reference: str | Path | None, verbose: bool = False) -> Path | None:
    """The reference's own sources, from the directory 'reference' when it
    holds them (the oracle's reference build; skipped when None or absent)."""
    if reference is None:
        return None
    ref = Path(reference)
    if not (ref / "src" / "calcul.cpp").exists() or shutil.which("make") is None:
        return None
    _run(["make", "-s", "-C", str(ROOT), "-f", "oracle/ref.mk", f"REF={ref}", f"-j{os.cpu_count() or 2}"])
    if verbose:
        print("built oracle/_ref")
    return ORACLE / "_ref"


def build_all(reference: str | Path | None = None, verbose: bool = False) -> None:
    """The library, the oracle and, given the reference's source directory,
    the reference build (default: the MCAC_REFERENCE environment variable)."""
    build_library(verbose)
    build_oracle(verbose)
    build_reference(reference if reference is not None else os.environ.get("MCAC_REFERENCE"), verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
