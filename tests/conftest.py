import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(REPO, "astronbodysim.jl_gb300")
for p in (REPO, PKG_ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def nb():
    """The astronbodysim package with libnbody_gb300.so loaded (built in place)."""
    import astronbodysim

    astronbodysim.load()
    return astronbodysim


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o

    o.lib()
    return o


@pytest.fixture(scope="session")
def golden():
    import json

    d = os.path.join(REPO, "tests", "golden")

    def load(name):
        with open(os.path.join(d, name)) as f:
            return json.load(f)

    return load
