import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    import __graft_entry__

    __graft_entry__.reference_env()
    from oracle import pyoracle

    pyoracle.build(ref=None)
    return pyoracle


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden.npz")))


@pytest.fixture(scope="session")
def glass():
    from pyglass_gb300 import build

    build.build()
    from pyglass_gb300 import glass as g

    return g


@pytest.fixture(scope="session")
def gpu(glass):
    if glass.device_count() == 0:
        pytest.fail("GPU test run without a visible CUDA device")
    return glass
