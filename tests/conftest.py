"""Shared fixtures.  `-m gpu` tests need a CUDA device and the built
libvdr.so; everything else runs on CPU."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libvdr.so")


@pytest.fixture(scope="session")
def vdr():
    """The product package (imported as vdr_gb300)."""
    return __graft_entry__.package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib(vdr):
    """libvdr.so, built for this host and loaded; fails (not skips) when the
    library cannot be built on a GPU machine."""
    if not _cuda_available():
        pytest.skip("no CUDA device")
    vdr.build_library()
    return vdr.load_library()
