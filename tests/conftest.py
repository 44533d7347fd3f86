"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device (a GB300); the rest run on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libsymeig.so")


@pytest.fixture(scope="session")
def pkg():
    """The product package (symmetriceigenproblem.jl_gb300), loaded by path."""
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure)."""
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def cuda(pkg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    pkg.load_library()
    return torch


def rotation_grid(pkg, rng, n, k, dtype=np.float64):
    """Julia-layout (n-1) x k grid of (cos t, sin t) with t ~ U[0, 2pi)."""
    th = rng.random((max(n - 1, 0), k)) * 2 * np.pi
    g = pkg.givens_buffer(max(n - 1, 0), k, dtype)
    g[..., 0] = np.cos(th)
    g[..., 1] = np.sin(th)
    return g


def to_device_colmajor(torch, A):
    """numpy column-major (m, n) -> CUDA tensor with the same column-major layout."""
    return torch.from_numpy(np.ascontiguousarray(A.T)).cuda().T
