import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as graft  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libddd_gb300.so")


@pytest.fixture(scope="session")
def pkg():
    return graft.load_package()


@pytest.fixture(scope="session")
def oracle():
    o, _ = graft.load_oracle()
    o.build()
    return o


@pytest.fixture(scope="session")
def fixtures():
    _, fx = graft.load_oracle()
    return fx


@pytest.fixture(scope="session")
def synth(pkg):
    import ddd_gb300.synth as s
    return s


@pytest.fixture(scope="session")
def ctx(pkg):
    """A GPU context; the library must already be built (build() runs before the GPU tests)."""
    return pkg.get_context(0)


def k5_of(dln, mat):
    return np.array([dln.coreRadSq, mat.μ4π, mat.μ8π, mat.μ4πν, mat.νμ4πν], dtype=np.float64)
