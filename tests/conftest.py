"""Shared pytest configuration.

Markers: ``gpu`` -- needs a CUDA device (run with ``-m gpu`` on a GB300);
everything else runs on the CPU.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def mak():
    """The package, with libmak_gb300.so built in-tree (no CPU fallback)."""
    import __graft_entry__ as ge

    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.fixture
def rng():
    return np.random.default_rng(123)


def to_dev(A, device):
    """numpy (m x n) -> column-major CUDA tensor."""
    import torch

    return torch.from_numpy(np.asfortranarray(A)).to(device).t().contiguous().t() \
        if A.ndim == 2 else torch.from_numpy(A).to(device)


def to_host(X):
    return X.detach().cpu().numpy()
