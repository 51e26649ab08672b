import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_SCENES = ["ico3", "ico4", "soup3k", "dups2k"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA kernels")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="session", params=GOLDEN_SCENES)
def golden(request):
    g = load_golden(request.param)
    g["name"] = request.param
    return g


@pytest.fixture(scope="session")
def lib_built():
    from sequoia_gb300 import _build
    return _build.build()


@pytest.fixture(scope="session")
def ctx(lib_built):
    import sequoia_gb300 as sq
    return sq.Context(0)
