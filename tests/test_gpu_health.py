"""Failure detection, injected on the host (no GPU fault, no device-side trap or wait).

The reference has no run-time detection; it only throws at set-up
(src/Solver/Solver.cpp:150-153, 201).  Here a state check ends every step and follows
every upload (kernels/health.cuh): a NaN/infinity, density <= 0 or pressure <= 0 in an
interior cell sets a health bit; strict mode turns the bits into the status of the call.
The bad inputs are made on the host: a NaN cell, a negative density, a negative
pressure, a ghost-only NaN, a strong rarefaction on which the Roe scheme itself
produces a negative pressure (the step is located with the oracle), wrong element
counts and an unknown mode.
"""
import ctypes

import numpy as np
import pytest

from _cases import random_state
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu

NONFINITE, DENSITY, PRESSURE = _abi.HEALTH_STATE_NONFINITE, _abi.HEALTH_STATE_DENSITY, _abi.HEALTH_STATE_PRESSURE


def kh_cfg(solver="EulerRoe", precision=_abi.FP64):
    return _abi.make_config(solver=solver, size=(40, 36), boundary="PERIODIC", limiter="MinMod",
                            integrator="RungeKutta4", precision=precision)


def kh_state(precision=_abi.FP64):
    s = ic.kelvin_helmholtz(size=(40, 36), seed=5).reshape(36, 40, 4).copy()
    return s.astype(np.float32) if precision == _abi.FP32 else s


def state_bits(u, n):
    """The check of kernels/health.cuh restated in numpy on the interior cells (1D-3D
    states reshaped to (cells, n) by the caller)."""
    fin = np.all(np.isfinite(u), axis=1)
    out = NONFINITE if not fin.all() else 0
    rho, E = u[:, 0], u[:, -1]
    m2 = u[:, 1] * u[:, 1]
    for j in range(2, n - 1):
        m2 = m2 + u[:, j] * u[:, j]
    with np.errstate(invalid="ignore", over="ignore"):
        if np.any(fin & ~(rho > 0)):
            out |= DENSITY
        if np.any(fin & (rho > 0) & ~((2 * (rho * E)) > m2)):
            out |= PRESSURE
    return out


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC", "EulerHLL"])
@pytest.mark.parametrize("precision", [_abi.FP64, _abi.FP32])
def test_valid_run_is_healthy(hg, solver, precision):
    s = hg.Solver(kh_cfg(solver, precision))
    s.set_health_mode(_abi.HEALTH_STRICT)
    s.resetState(kh_state(precision))
    for _ in range(5):
        s.update(1)                      # strict: raises on any state bit
    assert s.health() == 0
    s.close()


@pytest.mark.parametrize("what,bit,status", [
    ("nan", NONFINITE, _abi.ERR_NONFINITE),
    ("inf", NONFINITE, _abi.ERR_NONFINITE),
    ("negative_density", DENSITY, _abi.ERR_UNPHYSICAL),
    ("zero_density", DENSITY, _abi.ERR_UNPHYSICAL),
    ("negative_pressure", PRESSURE, _abi.ERR_UNPHYSICAL),
])
@pytest.mark.parametrize("precision", [_abi.FP64, _abi.FP32])
def test_corrupted_upload(hg, what, bit, status, precision):
    u = kh_state(precision)
    y, x = 17, 23                                   # an interior cell
    if what == "nan":
        u[y, x, 2] = np.nan
    elif what == "inf":
        u[y, x, 3] = -np.inf
    elif what == "negative_density":
        u[y, x, 0] = -u[y, x, 0]
    elif what == "zero_density":
        u[y, x, 0] = -0.0
    else:                                            # E below the kinetic energy
        u[y, x, 3] = .5 * (u[y, x, 1] ** 2 + u[y, x, 2] ** 2) / u[y, x, 0] * .5
    s = hg.Solver(kh_cfg(precision=precision))
    s.resetState(u)                                  # record mode: the upload's bits are kept
    assert s.health() == bit
    s.set_health_mode(_abi.HEALTH_STRICT)
    with pytest.raises(hg.HgpuError) as e:
        s.resetState(u)
    assert e.value.status == status
    assert s.health() == bit                         # strict mode leaves the bits set until read
    assert s.health() == 0
    s.close()


def test_ghost_only_nan_is_not_flagged(hg):
    u = kh_state()
    u[0, 5, 0] = np.nan                              # a ghost cell: the step's fill overwrites it
    s = hg.Solver(kh_cfg())
    s.set_health_mode(_abi.HEALTH_STRICT)
    s.resetState(u)
    s.update(2)
    assert s.health() == 0
    s.close()


def test_health_off_skips_the_check(hg):
    u = kh_state()
    u[17, 23, 0] = np.nan
    s = hg.Solver(kh_cfg())
    s.set_health_mode(_abi.HEALTH_OFF)
    s.resetState(u)
    s.update(1, want_dt=False)
    assert s.health() & (NONFINITE | DENSITY | PRESSURE) == 0
    k_off = s.kernels_per_step()
    s.set_health_mode(_abi.HEALTH_RECORD)
    s.resetState(kh_state())
    s.update(1, want_dt=False)
    assert s.kernels_per_step() == k_off + 1         # the check is one kernel per step
    assert s.health() == 0
    with pytest.raises(hg.HgpuError) as e:
        s.set_health_mode(7)
    assert e.value.status == _abi.ERR_ARG
    s.close()


def rarefaction(n=128):
    """Two streams leaving each other at Mach ~11 (rho 1, p 0.1, u = -3 | +3): the
    linearised Roe flux gives a negative pressure at the centre within a few steps."""
    cfg = _abi.make_config(solver="EulerRoe", size=(n,), xmin=(0.,), xmax=(1.,), boundary="FREEFLOW",
                           limiter="Superbee", integrator="ForwardEuler", cfl=.5)
    x = ic.cell_centers((n,), (0.,), (1.,))[0].reshape(1, 1, n)
    st = ic.build_state_euler(1, 1.4, np.ones_like(x), np.where(x < .5, -3., 3.), 0., 0., np.full_like(x, .1))
    return cfg, st.reshape(-1)


def test_step_that_goes_unphysical(hg, oracle_mod):
    cfg, u0 = rarefaction()
    ref = oracle_mod.Oracle(cfg)
    ref.set_state(u0)
    s = hg.Solver(cfg)
    s.resetState(u0)
    first_bad = None
    for k in range(1, 9):
        ref.update(1)
        want = state_bits(ref.get_state().reshape(-1, 3)[2:-2], 3)
        s.update(1)
        got = s.health() & (NONFINITE | DENSITY | PRESSURE)
        assert got == want, "step %d: %d vs %d" % (k, got, want)   # the bits the oracle's state gives
        if want and first_bad is None:
            first_bad = k
    s.close()
    assert first_bad is not None and first_bad <= 6
    # strict mode: every step before the failure returns OK, the failing one the status
    s = hg.Solver(cfg)
    s.set_health_mode(_abi.HEALTH_STRICT)
    s.resetState(u0)
    for k in range(1, first_bad):
        s.update(1)
    with pytest.raises(hg.HgpuError) as e:
        s.update(1)
    assert e.value.status in (_abi.ERR_UNPHYSICAL, _abi.ERR_NONFINITE)
    s.close()


def test_batch_flags_only_the_corrupted_problem(hg):
    cfgs = [_abi.make_config(solver="EulerRoe", size=(24 + 8 * p, 20), boundary="FREEFLOW", limiter="Superbee",
                             integrator="RungeKutta2") for p in range(3)]
    b = hg.Batch(cfgs)
    for p, c in enumerate(cfgs):
        u = random_state(c, seed=p).reshape(20, c.size[0], 4).copy()
        if p == 1:
            u[10, 7, 0] = np.nan
        b.set_state(p, u.reshape(-1))
    b.update(1)
    flags = b.problem_health()
    assert list(flags & (NONFINITE | DENSITY | PRESSURE)) == [0, NONFINITE, 0]
    assert b.health() & NONFINITE
    assert list(b.problem_health()) == [0, 0, 0]   # read clears
    b.close()


def test_wrong_counts_and_handles(hg):
    cfg = kh_cfg()
    s = hg.Solver(cfg)
    L = hg.lib()
    u = kh_state().reshape(-1)
    n = u.size
    assert L.hgpu_set_state(s.h, u.ctypes.data, n - 1) == _abi.ERR_ARG
    assert L.hgpu_get_state(s.h, u.ctypes.data, n + 4) == _abi.ERR_ARG
    assert L.hgpu_update_host(s.h, u.ctypes.data, n, 1, u.ctypes.data, n - 4, None) == _abi.ERR_ARG
    assert L.hgpu_update_host(s.h, u.ctypes.data, n, 0, u.ctypes.data, n, None) == _abi.ERR_ARG
    assert L.hgpu_set_state_potential(s.h, u.ctypes.data, n, u.ctypes.data, 3) == _abi.ERR_ARG
    assert L.hgpu_update(s.h, -1, None) == _abi.ERR_ARG
    assert L.hgpu_set_state(None, u.ctypes.data, n) == _abi.ERR_ARG
    s.close()
    cfgs = [_abi.make_config(solver="EulerRoe", size=(24, 20), integrator="RungeKutta2")] * 2
    b = hg.Batch(cfgs)
    x = np.zeros(24 * 20 * 4)
    assert L.hgpu_batch_set_state(b.h, 0, x.ctypes.data, x.size - 1) == _abi.ERR_ARG
    assert L.hgpu_batch_set_state(b.h, 2, x.ctypes.data, x.size) == _abi.ERR_OOB
    flags = (ctypes.c_uint32 * 3)()
    assert L.hgpu_batch_problem_health(b.h, flags, 3) == _abi.ERR_ARG
    b.close()
