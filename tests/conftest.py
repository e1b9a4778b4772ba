"""pytest configuration: the `gpu` marker and shared fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_files():
    return sorted(GOLDEN.glob("golden_*.npz"))


def options_files():
    """Fixtures of the reference with non-default scheme switches."""
    return sorted(GOLDEN.glob("options_*.npz"))


@pytest.fixture(scope="session")
def cuda_available():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True
