"""The C ABI on the CPU: libbehf.so builds, loads without a GPU, and exports every function that
include/behf.h declares (no compute call is made)."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "behf.h"


def declared() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(behf_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_api():
    names = declared()
    for must in ("behf_create", "behf_set_medium", "behf_run", "behf_get_seismograms", "behf_gradient",
                 "behf_misfit_gradient", "behf_autotune", "behf_run_batch", "behf_field_norm_noalloc"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from behf import build
    lib = ctypes.CDLL(str(build.build()))
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    lib.behf_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.behf_version()


def test_errors_without_a_context():
    from behf import build
    lib = ctypes.CDLL(str(build.build()))
    lib.behf_last_error.restype = ctypes.c_char_p
    assert lib.behf_run(None, 1) == -1
    assert b"null" in lib.behf_last_error()
    assert lib.behf_get_info(None, None) == -1
    assert lib.behf_run_batch(None, 1, 1) == -1
