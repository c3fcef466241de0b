import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bluebottle-3.0_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def bbpp_lib():
    """Build (if needed) and load libbbpp.so."""
    import bbpp
    if not os.path.exists(bbpp.LIBPATH):
        import build
        build.build()
    return bbpp.lib()


@pytest.fixture(scope="session")
def orc():
    import pyoracle
    pyoracle.build()
    return pyoracle
