"""Test configuration: paths to the library binding and the oracle, the `gpu`
marker, and shared fixtures."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpu-bundle-adjustment_gb300"
sys.path.insert(0, str(PKG))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


def _ensure_built():
    sys.path.insert(0, str(PKG))
    import build as gba_build  # noqa: E402

    gba_build.build()


@pytest.fixture(scope="session")
def gba():
    _ensure_built()
    import gba_gb300

    return gba_gb300


@pytest.fixture(scope="session")
def oracle():
    import oracle as oracle_mod

    return oracle_mod


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)
