"""Shared test setup: import paths, the ``gpu`` marker and common fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fwi2dacoustic-mpi-lbfgs_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) device")


@pytest.fixture(scope="session")
def oracles():
    import oracle as O
    O.build()
    return O, O.Oracle("f32"), O.Oracle("f64")


@pytest.fixture(scope="session")
def engine_lib():
    import build as B
    B.build()
    import fwigpu
    return fwigpu.load_library()


def ricker(nt, dt, f0, t0=None):
    t0 = 1.2 / f0 if t0 is None else t0
    a = (np.pi * f0 * (np.arange(nt) * dt - t0)) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)
