"""Shared test set-up: import paths, the ``gpu`` marker, and small problem builders."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "mixed-precision-optimization-method_gb300"
for p in (str(ROOT), str(PKG_DIR)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def behf_lib():
    """The CUDA library, built in-tree; GPU tests fail loudly if it cannot be built or loaded."""
    from behf import build
    import behf
    build.build()
    return behf.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    return pyoracle


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}
