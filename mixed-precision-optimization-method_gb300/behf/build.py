"""Build libbehf.so for sm_103a with nvcc (in-tree, no CMake).

Each translation unit of ``csrc/`` is compiled in parallel to ``_build/``, then linked with
``nvcc -shared`` into ``behf/_lib/libbehf.so``.  ``kernels_aux.cu`` is compiled with
``-fmad=false`` so that the double-precision coefficient build rounds like a host computation.
Usage: ``python -m behf.build`` (from the package directory) or ``behf.build.build()``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent                      # mixed-precision-optimization-method_gb300/
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
BUILD = ROOT / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libbehf.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-I", str(CSRC), "-I", str(INCLUDE)]
PER_FILE = {"kernels_aux.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None,
          lib: Path | None = None, objdir: Path | None = None) -> Path:
    """Compile (incrementally) and return the path of libbehf.so.

    lib / objdir redirect the output (a build with different compile-time options next to the in-tree one)."""
    LIB = Path(lib) if lib else globals()["LIB"]
    BUILD = Path(objdir) if objdir else globals()["BUILD"]
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    headers = _headers()
    objs = []
    jobs = []
    for src in _sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers, Path(__file__)]):
            cmd = [cc, *ARCH, *NVFLAGS, *PER_FILE.get(src.name, []), *(extra or []), "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, LIB)
    return LIB


DRIVER_SRC = ROOT / "driver" / "behf_main.cpp"
DRIVER = LIBDIR / "behf_run"


def cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("no C++ compiler found")


def build_driver(force: bool = False, verbose: bool = False) -> Path:
    """Compile the command-line driver (host C++ only) against libbehf.so; the binary finds the library
    next to itself (rpath $ORIGIN)."""
    lib = build(verbose=verbose)
    if force or _stale(DRIVER, [DRIVER_SRC, INCLUDE / "behf.h", lib, Path(__file__)]):
        tmp = DRIVER.with_name(DRIVER.name + ".tmp")
        cmd = [cxx(), "-std=c++17", "-O2", "-Wall", "-I", str(INCLUDE), str(DRIVER_SRC), "-o", str(tmp),
               "-L", str(LIBDIR), "-lbehf", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
    print(build_driver(force="--force" in sys.argv, verbose=True))
