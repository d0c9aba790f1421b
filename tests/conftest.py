import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libRobotecGPULidar.so")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture
def rgl():
    """The C API through ctypes; every test starts and ends with rgl_cleanup() like the reference's
    RGLTest fixture (test/include/helpers/commonHelpers.hpp:32-38)."""
    from robotecgpulidar_gb300 import rgl as api

    lib = api.lib()
    api.check(lib.rgl_configure_logging(api.RGL_LOG_LEVEL_OFF, None, False))
    api.check(lib.rgl_cleanup())
    yield api
    api.check(lib.rgl_cleanup())
