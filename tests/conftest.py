"""Shared fixtures.  Tests marked `gpu` need a CUDA device and the built
libdtsgb.so; everything else runs on the CPU."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libdtsgb.so")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def dts():
    """The product package (loads libdtsgb.so, building it if needed)."""
    import __graft_entry__
    __graft_entry__.build()
    import domain_transform_solver_gb300 as D
    return D


@pytest.fixture(scope="session")
def gpu_ready(dts):
    import ctypes
    n = ctypes.c_int()
    cudart = None
    try:
        import torch
        ok = torch.cuda.is_available()
    except Exception:
        ok = False
    if not ok:
        pytest.skip("no CUDA device")
    return dts
