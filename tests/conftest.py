"""Shared test setup: repo on sys.path, the `gpu` marker, golden-fixture loading."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a) and the built library")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        with np.load(GOLDEN / f"{name}.npz") as z:
            return {k: z[k] for k in z.files}
    return load


@pytest.fixture(scope="session")
def lib():
    """The C-ABI library, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    from jscc_recon_spect_cylinder_gb300 import _lib
    return _lib.load(build_if_missing=True)


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("GPU tests need CUDA; run them on a GB300 (pytest -m gpu)")
    from jscc_recon_spect_cylinder_gb300 import _lib
    _lib.load(build_if_missing=True)
    return torch.device("cuda:0")


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
