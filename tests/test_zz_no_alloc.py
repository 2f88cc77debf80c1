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

CASES = [("EulerRoe", _abi.FP64, (96, 80), _abi.COMPAT_REF), ("EulerHLLC", _abi.FP64, (96, 80), _abi.COMPAT_REF),
         ("EulerRoe", _abi.FP32, (64, 72), _abi.COMPAT_REF), ("EulerHLLC", _abi.FP64, (24, 20, 18), _abi.COMPAT_REF),
         ("EulerHLL", _abi.FP64, (96, 80), _abi.COMPAT_REF), ("EulerHLL", _abi.FP32, (30, 26, 22), _abi.COMPAT_REF),
         ("EulerRoe", _abi.FP64, (200,), _abi.COMPAT_REF), ("EulerRoe", _abi.FP64, (20, 18, 16), _abi.COMPAT_REF),
         ("EulerHLLC", _abi.FP32, (64, 72), _abi.COMPAT_REF), ("EulerRoe", _abi.FP64, (96, 80), _abi.COMPAT_SEAM),
         ("EulerHLLC", _abi.FP64, (96, 80), _abi.COMPAT_SEAM)]


def initial_state(size, dtype):
    if len(size) == 1:
        return ic.sod(size=size, dtype=dtype)
    if len(size) == 2:
        return ic.kelvin_helmholtz(size=size, seed=5, dtype=dtype)
    return ic.lognormal_grf(size=size, corr_cells=3.0, seed=6, gamma=1.4, dtype=dtype)


@pytest.mark.parametrize("solver,precision,size,compat", CASES)
def test_noalloc_dt_matches_solver_dt_twice(hg, solver, precision, size, compat):
    boundary = {1: "FREEFLOW", 2: "PERIODIC", 3: "MIRROR"}[len(size)]
    cfg = _abi.make_config(solver=solver, size=size, boundary=boundary, limiter="MinMod",
                           integrator="ForwardEuler", cfl=.5, precision=precision, compat=compat)
    dtype = np.float32 if precision == _abi.FP32 else np.float64
    init = initial_state(size, dtype)
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


def device_free_bytes():
    """Free bytes of the current device (cuMemGetInfo on the calling thread's context)."""
    cu = ctypes.CDLL("libcuda.so.1")
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert cu.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_noalloc_calls_leave_device_memory_unchanged(hg):
    """After the first call on the device (which loads the library's module holding the
    scratch array), further calls allocate nothing: the device's free memory stays
    the same over them."""
    cfg = _abi.make_config(solver="EulerRoe", size=(256, 200), boundary="PERIODIC", limiter="MinMod",
                           integrator="ForwardEuler")
    s = hg.Solver(cfg)
    s.resetState(ic.kelvin_helmholtz(size=(256, 200), seed=2))
    s.update(1)
    L = hg.lib()
    dt = ctypes.c_double()
    args = (ctypes.byref(cfg), ctypes.c_void_p(s.state_device_ptr()), ctypes.byref(dt), ctypes.c_void_p(s.stream()))
    assert L.hgpu_cfl_timestep_noalloc(*args) == 0
    before = device_free_bytes()
    values = set()
    for _ in range(20):
        assert L.hgpu_cfl_timestep_noalloc(*args) == 0
        values.add(dt.value)
    assert device_free_bytes() == before
    assert len(values) == 1
    s.close()


def test_noalloc_uses_a_zero_potential(hg):
    """The entry point takes no potential: its dt is the zero-potential one.  For a
    state that a solver steps with a nonzero static potential it is the dt that state
    has without the potential (the documented behaviour), not the solver's.  State and
    potential are periodic images of their interiors, so the device state's ghost cells
    are what the step's ghost fill would write."""
    size = (48, 40)
    cfg = _abi.make_config(solver="EulerRoe", size=size, boundary="PERIODIC", limiter="MinMod",
                           integrator="ForwardEuler")

    def periodic(a):
        a = a.reshape(size[1], size[0], -1)[2:-2, 2:-2]
        return np.pad(a, ((2, 2), (2, 2), (0, 0)), mode="wrap").reshape(-1)

    u = periodic(ic.kelvin_helmholtz(size=size, seed=8))
    phi = periodic(ic.smooth_perturbation(size, seed=9, amp=.5))
    grav, plain = hg.Solver(cfg), hg.Solver(cfg)
    grav.resetState(u, potential=phi)
    L = hg.lib()
    dt = ctypes.c_double()
    assert L.hgpu_cfl_timestep_noalloc(ctypes.byref(cfg), ctypes.c_void_p(grav.state_device_ptr()),
                                       ctypes.byref(dt), ctypes.c_void_p(grav.stream())) == 0
    plain.resetState(grav.getState())
    zero_potential_dt = plain.update(1)
    with_potential_dt = grav.update(1)
    assert dt.value == zero_potential_dt
    assert with_potential_dt != zero_potential_dt
    plain.close()
    grav.close()


def test_noalloc_rejects_grids_beyond_its_scratch(hg):
    cfg = _abi.make_config(solver="EulerRoe", size=(4100, 4100))
    dt = ctypes.c_double()
    L = hg.lib()
    dummy = ctypes.c_double(0.0)  # never read: the size check comes first
    st = L.hgpu_cfl_timestep_noalloc(ctypes.byref(cfg), ctypes.cast(ctypes.pointer(dummy), ctypes.c_void_p),
                                     ctypes.byref(dt), None)
    assert st == 5  # HGPU_ERR_OOB
    assert "exceeds the fixed scratch limit" in L.hgpu_last_error().decode()
