"""A malformed hgpu_config is refused by hgpu_create / hgpu_batch_create with
HGPU_ERR_CONFIG and a message, before any device work (so these run without a GPU).
The reference throws at set-up for the cases it checks at all: no size information
(src/HydroGPUApp.cpp:214-222), an unknown integrator (src/Solver/Solver.cpp:201), an
unknown solver (src/HydroGPUApp.cpp:346-348), an unknown boundary method (:509)."""
import ctypes
import math

import pytest

from hydrodynamicsgpu_gb300 import _abi


def cfg_with(**field_values):
    c = _abi.make_config(solver="EulerRoe", size=(32, 24), boundary="PERIODIC", limiter="MinMod",
                         integrator="RungeKutta2")
    for k, v in field_values.items():
        if k == "size":
            for i in range(3):
                c.size[i] = v[i]
        elif k == "boundary":
            c.boundary[v[0]][v[1]] = v[2]
        elif k == "xmax":
            for i in range(3):
                c.xmax[i] = v[i]
        else:
            setattr(c, k, v)
    return c


BAD = [
    ("no active axis", dict(size=(1, 1, 1))),
    ("axis below 5 cells", dict(size=(4, 24, 1))),
    ("size beyond dim", dict(dim=1)),
    ("dim 4", dict(dim=4)),
    ("solver 3", dict(solver=3)),
    ("solver -1", dict(solver=-1)),
    ("limiter 20", dict(limiter=20)),
    ("limiter -2", dict(limiter=-2)),
    ("integrator 12", dict(integrator=12)),
    ("precision 2", dict(precision=2)),
    ("compat 2", dict(compat=2)),
    ("boundary 3", dict(boundary=(0, 1, 3))),
    ("boundary -2", dict(boundary=(1, 0, -2))),
    ("gamma 1", dict(gamma=1.0)),
    ("gamma NaN", dict(gamma=math.nan)),
    ("cfl 0", dict(cfl=0.0)),
    ("cfl NaN", dict(cfl=math.nan)),
    ("fixed dt -1", dict(use_fixed_dt=1, fixed_dt=-1.0)),
    ("xmax = xmin", dict(xmax=(-.5, .5, .5))),
    ("negative relaxations", dict(gauss_seidel_max_iter=-3)),
]


@pytest.mark.parametrize("name,fields", BAD, ids=[b[0] for b in BAD])
def test_create_refuses(hg, name, fields):
    c = cfg_with(**fields)
    h = ctypes.c_void_p()
    st = hg.lib().hgpu_create(ctypes.byref(c), ctypes.byref(h))
    assert st == _abi.ERR_CONFIG, (name, st)
    assert hg.lib().hgpu_last_error().decode()
    arr = (_abi.HgpuConfig * 2)(cfg_with(), c)
    assert hg.lib().hgpu_batch_create(arr, 2, ctypes.byref(h)) == _abi.ERR_CONFIG


def test_null_arguments(hg):
    h = ctypes.c_void_p()
    assert hg.lib().hgpu_create(None, ctypes.byref(h)) == _abi.ERR_ARG
    c = cfg_with()
    assert hg.lib().hgpu_create(ctypes.byref(c), None) == _abi.ERR_ARG
    assert hg.lib().hgpu_set_health_mode(None, 1) == _abi.ERR_ARG


def test_host_side_sizes_refused_before_device_work(hg):
    """Counts and sizes the host can check are refused before any device call: an
    empty or negative batch, and a grid beyond the allocation-free timestep's fixed
    scratch (its pointer is never read)."""
    h = ctypes.c_void_p()
    arr = (_abi.HgpuConfig * 1)(cfg_with())
    assert hg.lib().hgpu_batch_create(arr, 0, ctypes.byref(h)) == _abi.ERR_ARG
    assert hg.lib().hgpu_batch_create(arr, -3, ctypes.byref(h)) == _abi.ERR_ARG
    big = _abi.make_config(solver="EulerRoe", size=(4100, 4100))
    dt = ctypes.c_double()
    dummy = ctypes.c_double(0.)
    assert hg.lib().hgpu_cfl_timestep_noalloc(ctypes.byref(big), ctypes.cast(ctypes.pointer(dummy), ctypes.c_void_p),
                                              ctypes.byref(dt), None) == _abi.ERR_OOB
