"""Shared test setup: the `gpu` marker, the repository on sys.path, builds.

Tests marked `gpu` need a GB300 and the in-tree libwedg.so; everything else
runs on the CPU (the oracle, the host-side precompute, the C ABI's exports).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libwedg.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import rhs
    rhs.build()
    return rhs


@pytest.fixture(scope="session")
def wedg_lib():
    from edg_westervelt_gb300 import build
    build.build()
    from edg_westervelt_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def gpu(wedg_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    return torch.device("cuda:0")


def rel_max(a, b):
    """Max-norm relative difference of the RHS pairs (ut, vt), as test/runtests.jl:228-229."""
    import numpy as np
    return max(float(np.max(np.abs(a[0] - b[0])) / np.max(np.abs(a[0]))),
               float(np.max(np.abs(a[1] - b[1])) / np.max(np.abs(a[1]))))
