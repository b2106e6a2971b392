import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Make sure the native libraries exist (build() is normally run before the tests)."""
    from eig_gb300 import build as B
    need = [os.path.join(B.LIB, "libgpupca.so"), os.path.join(B.LIB, "libgpsynth.so"),
            os.path.join(B.ORACLE_BIN, "liboracle.so")]
    if not all(os.path.exists(p) for p in need):
        B.build()
    return True


@pytest.fixture(scope="session")
def gpu():
    from eig_gb300 import native
    h = native.Handle(0)
    yield h
    h.close()
