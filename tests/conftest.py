import ctypes
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libhgpu.so")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def oracle_mod():
    import pyoracle
    pyoracle.build_oracle()
    return pyoracle


@pytest.fixture(scope="session")
def hg():
    import hydrodynamicsgpu_gb300 as hg
    hg.lib()
    return hg


@pytest.fixture(autouse=True)
def _checked_build_findings(request):
    """Under the checked library (HGPU_EXPECT_CHECKED set, tests/test_gpu_checked.py),
    every GPU test ends by reading the index tests' word and the guard bands of every
    live device buffer: both must be clean."""
    yield
    if os.environ.get("HGPU_EXPECT_CHECKED") and request.node.get_closest_marker("gpu"):
        import hydrodynamicsgpu_gb300 as hg
        f = ctypes.c_uint32()
        st = hg.lib().hgpu_checked_status(ctypes.byref(f))
        assert st == 0, "not the checked library: %d" % st
        assert f.value == 0, "checked build: %s" % hg.lib().hgpu_last_error().decode()
