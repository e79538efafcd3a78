"""Build recipe for the oracle (test infrastructure, the checker of the CUDA path).

* ``build_oracle()`` compiles ``behf_oracle.cpp`` (forward) and ``behf_adjoint.cpp`` (FP64 discrete
  adjoint) into ``oracle/_build/liboracle.so``.
* ``build_ref()`` compiles the reference's own kernel bodies for the CPU into
  ``oracle/_ref/libbehf_ref.so``, linked with the reference's ``outputfunc.cpp`` (compiled
  where it lies) for its medium builder ``create_model_all``.  It reads ``kernel.cu`` from the reference tree, copies the
  text of ``Source``, ``FD_Vbottom`` and ``FD_Tbottom`` and the ``d_C*`` scale macros into
  ``oracle/_ref/ref_kernels.inc`` (git-ignored: reference source never enters the repository)
  and compiles it with ``ref_harness.cpp``.  It is only possible where the reference tree
  exists; elsewhere the committed fixtures under ``tests/golden`` stand in for it.

Both use ``-ffp-contract=off`` so that x86 and Arm hosts round identically.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# The read-only reference checkout: BEHF_REFERENCE_TREE, else a directory named "reference" beside this repository
# (where the build container mounts it; the GPU machines have none and use the committed fixtures).
REFERENCE_TREE = Path(os.environ.get("BEHF_REFERENCE_TREE") or HERE.parent.parent / "reference")

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def _needs(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "liboracle.so"
    srcs = [HERE / "behf_oracle.cpp", HERE / "behf_adjoint.cpp"]
    deps = [*srcs, HERE / "behf_oracle.h"]
    if force or _needs(out, deps):
        cmd = ["g++", *CXXFLAGS, "-o", str(out), *map(str, srcs)]
        subprocess.run(cmd, check=True)
    return out


def _extract_function(src: str, name: str) -> str:
    m = re.search(r"__global__\s+void\s+" + re.escape(name) + r"\s*\(", src)
    if not m:
        raise RuntimeError(f"kernel {name} not found in kernel.cu")
    i = src.index("{", m.end())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[m.start(): j + 1]
    raise RuntimeError(f"unbalanced braces in {name}")


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference kernels for the CPU; None if the reference tree is absent."""
    kernel_cu = REFERENCE_TREE / "kernel.cu"
    if not kernel_cu.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "libbehf_ref.so"
    inc = REF_OUT / "ref_kernels.inc"
    deps = [kernel_cu, REFERENCE_TREE / "outputfunc.cpp", HERE / "ref_harness.cpp", Path(__file__)]
    if force or _needs(out, deps):
        src = kernel_cu.read_text(encoding="latin-1")
        macros = [ln for ln in src.splitlines() if re.match(r"#define\s+d_C\w+\s", ln)]
        parts = ["// generated by oracle/build.py from the reference kernel.cu -- do not commit"]
        parts += macros
        for name in ("Source", "FD_Vbottom", "FD_Tbottom"):
            parts.append(_extract_function(src, name))
        inc.write_text("\n".join(parts) + "\n")
        cmd = ["g++", *CXXFLAGS, "-w", "-I", str(REF_OUT), "-I", str(REFERENCE_TREE), "-o", str(out),
               str(HERE / "ref_harness.cpp"), str(REFERENCE_TREE / "outputfunc.cpp")]
        subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
