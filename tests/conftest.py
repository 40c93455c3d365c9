import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "polyq-v1.0_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native():
    """The built native library (compiled on first use)."""
    from polyq_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def gpu(native):
    from polyq_gb300 import _native
    _native.check(native.pq_init(0))
    return native
