"""Conserved totals on periodic domains, and the FP32 error against FP64.

With the SEAM scheme (eigenbasis and Delta-q-tilde on every face between grid cells,
ghost refresh per stage) the fluxes at the two periodic seam faces coincide, so the
interior totals of rho, m and E change only by round-off.  The REF scheme reproduces
the reference, whose Delta-q-tilde at faces 1 and SIZE-1 stays zero: its seam faces
differ and the totals drift (measured here, not asserted small)."""
import numpy as np
import pytest

from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu


def totals(state, size, n):
    u = state.reshape(size[1], size[0], n)[2:-2, 2:-2]
    return u.reshape(-1, n).sum(0), np.abs(u).reshape(-1, n).sum(0)


@pytest.mark.parametrize("integrator", ["ForwardEuler", "RungeKutta2", "RungeKutta4", "RungeKutta3TVD"])
@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC"])
def test_seam_scheme_conserves_totals(hg, solver, integrator):
    size = (68, 68)
    cfg = _abi.make_config(solver=solver, size=size, boundary="PERIODIC", limiter="MinMod", integrator=integrator,
                           compat=_abi.COMPAT_SEAM)
    s = hg.Solver(cfg)
    u0 = ic.kelvin_helmholtz(size=size, seed=4).reshape(-1)
    s.resetState(u0)
    t0, scale = totals(u0, size, 4)
    s.update(20)
    t1, _ = totals(s.getState(), size, 4)
    drift = np.abs(t1 - t0) / scale
    assert np.all(drift <= 1e-13), drift
    s.close()


def test_ref_scheme_seam_drift_is_measurable(hg):
    """The reference's own scheme is not conservative at the periodic seam."""
    size = (68, 68)
    cfg = _abi.make_config(solver="EulerRoe", size=size, boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4")
    s = hg.Solver(cfg)
    u0 = ic.kelvin_helmholtz(size=size, seed=4).reshape(-1)
    s.resetState(u0)
    t0, scale = totals(u0, size, 4)
    s.update(20)
    t1, _ = totals(s.getState(), size, 4)
    assert np.max(np.abs(t1 - t0) / scale) > 1e-12
    s.close()


def test_fp32_error_against_fp64(hg):
    """FP32 KH 256^2 RK4 after 100 steps against the same run in FP64 (each with its own
    CFL dt): the normwise relative difference per conserved variable stays below 1e-4."""
    size = (256, 256)
    u0 = ic.kelvin_helmholtz(size=size, seed=0).reshape(-1)
    out = {}
    for prec in (_abi.FP64, _abi.FP32):
        cfg = _abi.make_config(solver="EulerRoe", size=size, boundary="PERIODIC", limiter="MinMod",
                               integrator="RungeKutta4", precision=prec)
        s = hg.Solver(cfg)
        s.resetState(u0.astype(np.float32) if prec == _abi.FP32 else u0)
        s.update(100)
        out[prec] = s.getState().astype(np.float64).reshape(-1, 4)
        s.close()
    a, b = out[_abi.FP32], out[_abi.FP64]
    err = np.max(np.abs(a - b), axis=0) / np.max(np.abs(b), axis=0)
    assert np.all(err <= 1e-4), err
