"""Test configuration: markers and import paths.

GPU tests are marked ``gpu`` and call the CUDA library through its C ABI; the
rest run on CPU (oracle pins, host logic, library exports).
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "fluid-engine-dev_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def port():
    import oracle
    o = oracle.port()
    o.set_threads(0)
    return o


@pytest.fixture(scope="session")
def reference():
    """The reference compiled from its own sources, where they exist."""
    import oracle
    try:
        r = oracle.reference()
    except Exception:
        r = None
    if r is None:
        pytest.skip("reference sources not present on this machine")
    r.set_threads(0)
    return r


def golden(name):
    import numpy as np
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.fail(f"missing golden fixture {name}")
    return dict(np.load(path, allow_pickle=False))
