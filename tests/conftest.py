"""Test configuration: the ``gpu`` marker and shared fixtures.

Tests marked ``gpu`` need a CUDA device and the built library; the rest run on
CPU only (oracle vs golden vectors, event builders, host logic, the C ABI's
exports).
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def golden():
    """Loader of the committed reference fixtures (tests/golden/*.npz)."""

    def load(name: str):
        return np.load(GOLDEN / f"{name}.npz")

    return load


@pytest.fixture(scope="session")
def built_library():
    """Build (incrementally) and load the CUDA library once per session."""
    from torchsim_gb300 import _build, _native

    _build.build()
    return _native.library()


@pytest.fixture(scope="session")
def cuda(built_library):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)
