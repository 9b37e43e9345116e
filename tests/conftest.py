"""Shared fixtures. CPU tests need no GPU; tests marked `gpu` need an sm_103 device."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "italy-rs_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import build_oracle
    if build_oracle.build_ref() is None:
        pytest.skip("the reference tree is not available on this machine")
    from oracle.oracle import Reference
    return Reference()


@pytest.fixture(scope="session")
def lib():
    import build as pkg_build  # italy-rs_gb300/build.py
    pkg_build.build()
    import sdfb
    return sdfb.load()


@pytest.fixture(scope="session")
def ctx(lib):
    import sdfb
    c = sdfb.Context(0)
    yield c
    c.close()


def grid_of(arr):
    """(origin, voxel, (nx, ny, nz)) from a golden [ox, oy, oz, voxel, nx, ny, nz] row."""
    a = np.asarray(arr, np.float64)
    return (np.float32(a[0]), np.float32(a[1]), np.float32(a[2])), float(np.float32(a[3])), (
        int(a[4]), int(a[5]), int(a[6]))


def unpack(bits, n):
    return np.unpackbits(bits)[:n]
