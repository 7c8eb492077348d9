"""Shared fixtures.  GPU tests carry the `gpu` marker and run only on a GB300."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running (full-size workloads)")


@pytest.fixture(scope="session")
def built_lib():
    """libgbnesta.so, built in-tree if it is missing or stale."""
    from opencliper_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def ctx(built_lib):
    import opencliper_gb300 as g
    c = g.Context(0)
    yield c
    c.close()


def rel_l2(a, b) -> float:
    import numpy as np
    a = np.asarray(a).astype(np.complex128)
    b = np.asarray(b).astype(np.complex128)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
