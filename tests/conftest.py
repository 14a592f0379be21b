"""Shared pytest configuration: the ``gpu`` marker and common fixtures."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
if str(ROOT / "tests") not in sys.path:
    sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path through the C ABI)")


@pytest.fixture(scope="session")
def golden():
    return np.load(ROOT / "tests" / "golden" / "golden.npz")


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from ffsim_gb300 import _lib

    _lib.load()
    return torch.device("cuda")


# edge cases of python/ffsim/testing/testing.py:24-35
NORB_NELEC_CASES = [
    (0, (0, 0)), (1, (0, 0)), (1, (1, 0)), (1, (0, 1)), (1, (1, 1)), (2, (1, 1)), (2, (2, 2)),
    (3, (2, 1)), (3, (1, 2)), (4, (3, 2)),
]
