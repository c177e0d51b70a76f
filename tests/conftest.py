"""Shared fixtures.

Tests marked ``gpu`` need a CUDA device and call the CUDA path through the
C ABI (libglass_gb300.so via ctypes).  Everything else runs on the CPU: the
oracle against the golden vectors, host logic, and the library's exported
symbols.  A GPU test never skips silently when the library or the device is
missing: it fails, because the product path has no fallback.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = REPO / "tests" / "golden"
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libglass_gb300.so")


@pytest.fixture(scope="session")
def golden_integration():
    return np.load(GOLDEN / "integration.npz", allow_pickle=False)


@pytest.fixture(scope="session")
def golden_calibration():
    return np.load(GOLDEN / "calibration.npz", allow_pickle=False)


@pytest.fixture(scope="session")
def built_library():
    """Builds (incrementally) and returns the path of libglass_gb300.so."""
    from glass_gb300.build import build

    return build()


@pytest.fixture(scope="session")
def native(built_library):
    """The drop-in `_glass_cuda_native` module on a real GPU."""
    from glass_gb300 import native as load_native

    module = load_native()
    assert module.cuda_available(), "CUDA device required for gpu tests"
    return module
