"""Shared test setup.

Markers: ``gpu`` tests need a CUDA device and call the library through its C
ABI; every other test runs on the CPU (oracle checks, host logic, ABI surface).
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_small.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def port():
    import port as P  # oracle/port.py
    if not os.path.isfile(P.LIB_PATH):
        P.build()
    P.lib()
    return P


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def gpulib():
    """The CUDA library, built in-tree if it is missing."""
    from msbg_gb300 import build, gpu
    if not os.path.isfile(gpu.LIB_PATH):
        build.build()
    gpu.load_library()
    return gpu


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))
