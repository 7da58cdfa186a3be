import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import bind
    bind.build()
    return bind.load("oracle")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")

    def load(name):
        return dict(np.load(os.path.join(d, name + ".npz")))
    return load


@pytest.fixture(scope="session")
def ctx():
    """A librtx context on cuda:0 (GPU tests only)."""
    import rendertoy_gb300 as rt
    from rendertoy_gb300 import build
    build.build()
    c = rt.Context(0)
    yield c
    c.close()
