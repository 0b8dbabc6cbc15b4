"""Shared pytest setup: the `gpu` marker, import paths and GPU fixtures."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "mpi-msfec_gb300")
for p in (PKG, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu():
    """The msfec binding with a built library; fails loudly (no fallback)."""
    if not _cuda_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    import msfec_build
    msfec_build.build()
    import msfec
    msfec.load_library()
    return msfec
