"""hgpu_cfl_timestep_noalloc: the CFL timestep without any device allocation.

This entry point serves callers that cannot call cudaMalloc (a host that owns the
device-memory budget through its own pool, code where allocation is forbidden, a
plug-in host that only lends its buffers).  It must return exactly the dt the
regular path computes in Solver::update for the same state, call after call (the
scratch array it shares between calls has to be re-armed correctly).

After a ForwardEuler step the state's ghost cells are already boundary-filled (the
self-gravity pass refreshes them), so the next update's dt is the CFL timestep of
exactly that device state: the two entry points see identical inputs.
"""
import ctypes

import numpy as np
import pytest

from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu

CASES = [("EulerRoe", _abi.FP64, (96, 80)), ("EulerHLLC", _abi.FP64, (96, 80)),
         ("EulerRoe", _abi.FP32, (64, 72)), ("EulerHLLC", _abi.FP64, (24, 20, 18)),
         ("EulerHLL", _abi.FP64, (96, 80)), ("EulerHLL", _abi.FP32, (30, 26, 22))]


@pytest.mark.parametrize("solver,precision,size", CASES)
def test_noalloc_dt_matches_solver_dt_twice(hg, solver, precision, size):
    boundary = "PERIODIC" if len(size) == 2 else "MIRROR"
    cfg = _abi.make_config(solver=solver, size=size, boundary=boundary, limiter="MinMod",
                           integrator="ForwardEuler", cfl=.5, precision=precision)
    dtype = np.float32 if precision == _abi.FP32 else np.float64
    if len(size) == 2:
        init = ic.kelvin_helmholtz(size=size, seed=5, dtype=dtype)
    else:
        init = ic.lognormal_grf(size=size, corr_cells=3.0, seed=6, gamma=1.4, dtype=dtype)
    s = hg.Solver(cfg)
    s.resetState(init)
    s.update(1)
    L = hg.lib()
    for call in range(2):
        dt = ctypes.c_double()
        st = L.hgpu_cfl_timestep_noalloc(ctypes.byref(cfg), ctypes.c_void_p(s.state_device_ptr()),
                                         ctypes.byref(dt), ctypes.c_void_p(s.stream()))
        assert st == 0, L.hgpu_last_error().decode()
        expected = s.update(1)
        assert dt.value == expected, "call %d: no-alloc dt %r vs solver dt %r" % (call, dt.value, expected)
    s.close()


def test_noalloc_rejects_grids_beyond_its_scratch(hg):
    cfg = _abi.make_config(solver="EulerRoe", size=(4100, 4100))
    dt = ctypes.c_double()
    L = hg.lib()
    dummy = ctypes.c_double(0.0)  # never read: the size check comes first
    st = L.hgpu_cfl_timestep_noalloc(ctypes.byref(cfg), ctypes.cast(ctypes.pointer(dummy), ctypes.c_void_p),
                                     ctypes.byref(dt), None)
    assert st == 5  # HGPU_ERR_OOB
    assert "exceeds the fixed scratch limit" in L.hgpu_last_error().decode()
