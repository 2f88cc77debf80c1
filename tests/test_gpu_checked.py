"""The small-grid parity suites under the checked build of the library.

libhgpu_checked.so is the same sources compiled with HGPU_CHECKED: every cell index
a kernel body computes is tested against its grid (a violation is recorded in a
device word and the access skipped; nothing traps), and every device allocation has
guard bands of a fixed byte pattern on both sides.  compute-sanitizer is not
available for these runs, so this build stands in for it.  The reference's own
kernels show why such checks matter: its 1D ghost-cell kernels address cells past
the end of the state (res/Common.cl:97-194, launched with size.x work-items by
src/Solver/Solver.cpp:414-418).

The parity suites run in a child process on the checked library; after every test
conftest.py reads hgpu_checked_status, which must report no index violation and no
overwritten guard band, and the tests themselves compare with the oracle as usual."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
SUITES = ["test_gpu_parity.py", "test_gpu_batch.py", "test_gpu_fused.py", "test_gpu_health.py",
          "test_gpu_update_host.py", "test_gpu_output.py", "test_gpu_conservation.py"]


def test_parity_suites_under_checked_build():
    sys.path.insert(0, REPO)
    from hydrodynamicsgpu_gb300 import build
    lib = build.build(checked=True)
    env = dict(os.environ, HGPU_LIBRARY=lib, HGPU_EXPECT_CHECKED="1")
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
           "-k", "not 2048 and not kh_2048"] + [os.path.join(HERE, s) for s in SUITES]
    r = subprocess.run(cmd, cwd=REPO, env=env, capture_output=True, text=True, timeout=1800)
    tail = (r.stdout + r.stderr)[-4000:]
    assert r.returncode == 0, tail
    assert " passed" in r.stdout, tail


def test_checked_status_refused_by_the_normal_build(hg):
    import ctypes
    from hydrodynamicsgpu_gb300 import _abi
    if os.environ.get("HGPU_EXPECT_CHECKED"):
        pytest.skip("running on the checked library")
    f = ctypes.c_uint32()
    assert hg.lib().hgpu_checked_status(ctypes.byref(f)) == _abi.ERR_UNSUPPORTED
