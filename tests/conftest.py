import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (Blackwell, sm_103a build)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx():
    import rnng_gb300
    rnng_gb300.build.build()
    c = rnng_gb300.Context(0)
    yield c
    c.close()


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_points(g):
    if "x" in g:
        return g["x"]
    return g["x_u8"].astype(np.float32)
