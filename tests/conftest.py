"""Shared pytest configuration.

Tests marked ``gpu`` need a CUDA device and the in-tree libcpetgb.so; all
others run on a CPU-only machine.  The oracle library (oracle/liboracle.so) is
built on first use.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libcpetgb.so")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library; fails (does not skip) when it cannot be used."""
    import torch
    from pycpet_gb300 import build, _lib

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build.build_library()
    L = _lib.lib()
    assert _lib.device_sms() > 0
    return L
