"""Shared test setup: import paths, the `gpu` marker, and session fixtures."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "asfand-tmvp_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def kem():
    """The CUDA library and a context on cuda:0 (GPU tests only)."""
    import tmvpkem
    tmvpkem.build.build()
    ctx = tmvpkem.Context(0)
    yield tmvpkem, ctx
    ctx.close()


def golden(name):
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, name)))
