"""hgpu_update_host (upload, nsteps updates, download in one call, the copies in
bands overlapped with the first and last step) against hgpu_set_state +
hgpu_update + hgpu_get_state on the same input: the same bits, state and dt.

The overlapped form covers 2D/3D EulerRoe, EulerHLLC and EulerHLL without a fixed dt,
gravity or a static potential; the band count depends on the size along the slowest
axis (one band below 128 rows in 2D / 16 planes in 3D), so the sizes below take 1, 2,
4 and 16 bands.  The other configurations take the plain form."""
import numpy as np
import pytest

from _cases import describe_diff, random_state, same
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu


def reference_run(hg, cfg, init, nsteps):
    s = hg.Solver(cfg)
    try:
        s.resetState(init)
        dt = s.update(nsteps)
        return s.getState(), dt
    finally:
        s.close()


def check(hg, cfg, init, nsteps=1, pinned=False):
    ref, rdt = reference_run(hg, cfg, init, nsteps)
    s = hg.Solver(cfg)
    try:
        if pinned:
            src = hg.PinnedArray(s.count, s.dtype)
            dst = hg.PinnedArray(s.count, s.dtype)
            try:
                src.array[:] = init
                out, dt = s.update_host(src.array, nsteps, out=dst.array)
                out = out.copy()
            finally:
                src.free()
                dst.free()
        else:
            out, dt = s.update_host(init, nsteps)
        assert dt == rdt, (dt, rdt)
        assert same(out, ref), describe_diff(out, ref)
        # the solver holds the new state: a further step continues as after hgpu_update
        s.update(1)
        ref2, _ = reference_run(hg, cfg, init, nsteps + 1)
        assert same(s.getState(), ref2), describe_diff(s.getState(), ref2)
    finally:
        s.close()


@pytest.mark.parametrize("solver,nsteps", [("EulerRoe", 1), ("EulerRoe", 3), ("EulerHLLC", 2)])
def test_kh_2048_rk4(hg, solver, nsteps):
    cfg = _abi.make_config(solver=solver, size=(2048, 2048), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4")
    check(hg, cfg, ic.kelvin_helmholtz(size=(2048, 2048), seed=0).reshape(-1), nsteps, pinned=True)


CASES_2D = [
    # size, boundary, integrator, limiter, precision, compat
    ((20, 18), "PERIODIC", "RungeKutta4", "MinMod", _abi.FP64, _abi.COMPAT_REF),            # 1 band
    ((37, 150), "MIRROR", "RungeKutta2", "Superbee", _abi.FP64, _abi.COMPAT_REF),           # 1 band
    ((40, 300), "FREEFLOW", "RungeKutta3TVD", "VanLeer", _abi.FP64, _abi.COMPAT_REF),        # 2 bands, alpha 3/4
    ((33, 517), "PERIODIC", "ForwardEuler", "Koren", _abi.FP64, _abi.COMPAT_REF),            # 4 bands, FE
    ((48, 520), "MIRROR", "RungeKutta4", "MinMod", _abi.FP32, _abi.COMPAT_REF),              # 4 bands, FP32
    ((64, 300), "PERIODIC", "RungeKutta2Heun", "MonotizedCentral", _abi.FP64, _abi.COMPAT_SEAM),
]


@pytest.mark.parametrize("size,bnd,integ,lim,prec,compat", CASES_2D)
@pytest.mark.parametrize("nsteps", [1, 2])
def test_roe_2d(hg, size, bnd, integ, lim, prec, compat, nsteps):
    cfg = _abi.make_config(solver="EulerRoe", size=size, boundary=bnd, integrator=integ, limiter=lim,
                           precision=prec, compat=compat)
    check(hg, cfg, random_state(cfg, seed=7, blocky=True), nsteps)


@pytest.mark.parametrize("size,bnd,integ", [((10, 9, 40), "MIRROR", "RungeKutta2"),        # 2 bands
                                            ((12, 11, 70), "PERIODIC", "RungeKutta4"),     # 4 bands
                                            ((9, 8, 7), "FREEFLOW", "RungeKutta3TVD")])    # 1 band
def test_roe_3d(hg, size, bnd, integ):
    cfg = _abi.make_config(solver="EulerRoe", size=size, boundary=bnd, integrator=integ, limiter="MinMod")
    check(hg, cfg, random_state(cfg, seed=8), nsteps=2)


@pytest.mark.parametrize("solver,size,bnd,integ,prec", [
    ("EulerHLLC", (20, 18), "PERIODIC", "RungeKutta4", _abi.FP64),           # 1 band
    ("EulerHLLC", (64, 520), "MIRROR", "RungeKutta2", _abi.FP64),            # 4 bands
    ("EulerHLL", (40, 300), "FREEFLOW", "RungeKutta3TVD", _abi.FP64),        # 2 bands, alpha 3/4
    ("EulerHLLC", (33, 517), "PERIODIC", "ForwardEuler", _abi.FP32),         # 4 bands, FE, FP32
    ("EulerHLL", (10, 9, 40), "MIRROR", "RungeKutta2", _abi.FP64),           # 3D, 2 bands
    ("EulerHLLC", (12, 11, 70), "PERIODIC", "RungeKutta4", _abi.FP64),       # 3D, 4 bands
])
def test_hll_family(hg, solver, size, bnd, integ, prec):
    cfg = _abi.make_config(solver=solver, size=size, boundary=bnd, integrator=integ, limiter="MinMod",
                           precision=prec)
    check(hg, cfg, random_state(cfg, seed=13, blocky=True), nsteps=2)


def test_mixed_boundaries_per_side(hg):
    bnd = [("PERIODIC", "PERIODIC"), ("MIRROR", "FREEFLOW")]
    cfg = _abi.make_config(solver="EulerRoe", size=(30, 290), boundary=bnd, integrator="RungeKutta4")
    check(hg, cfg, random_state(cfg, seed=9), nsteps=2)


@pytest.mark.parametrize("kw", [dict(solver="EulerHLLC", size=(300,)),
                                dict(solver="EulerHLLC", size=(40, 300), use_fixed_dt=True, fixed_dt=1e-4),
                                dict(solver="EulerRoe", size=(300,)),
                                dict(solver="EulerRoe", size=(40, 300), use_fixed_dt=True, fixed_dt=1e-4),
                                dict(solver="EulerRoe", size=(40, 300), use_gravity=True,
                                     gauss_seidel_max_iter=3)])
def test_plain_form_configurations(hg, kw):
    cfg = _abi.make_config(boundary="PERIODIC", integrator="RungeKutta2", **kw)
    check(hg, cfg, random_state(cfg, seed=10), nsteps=2)


def test_in_place_buffer(hg):
    cfg = _abi.make_config(solver="EulerRoe", size=(40, 300), boundary="PERIODIC", integrator="RungeKutta4")
    init = random_state(cfg, seed=11)
    ref, rdt = reference_run(hg, cfg, init, 2)
    s = hg.Solver(cfg)
    buf = init.copy()
    out, dt = s.update_host(buf, 2, out=buf)
    s.close()
    assert out is buf and dt == rdt
    assert same(buf, ref), describe_diff(buf, ref)


def test_after_static_potential(hg):
    """A solver that ran with a static potential switches back to a zero potential, as
    hgpu_set_state does, and its captured step is rebuilt."""
    cfg = _abi.make_config(solver="EulerRoe", size=(40, 300), boundary="FREEFLOW", integrator="RungeKutta2")
    init = random_state(cfg, seed=12)
    pot = np.random.default_rng(3).uniform(-.1, .1, cfg.size[0] * cfg.size[1])
    s = hg.Solver(cfg)
    try:
        s.resetState(init, potential=pot)
        s.update(1)
        out, dt = s.update_host(init, 1)
        ref, rdt = reference_run(hg, cfg, init, 1)
        assert dt == rdt and same(out, ref), describe_diff(out, ref)
        s.update(1)
        ref2, _ = reference_run(hg, cfg, init, 2)
        assert same(s.getState(), ref2)
        assert not np.any(s.getPotential())
    finally:
        s.close()


def test_bad_arguments(hg):
    cfg = _abi.make_config(solver="EulerRoe", size=(20, 18))
    s = hg.Solver(cfg)
    try:
        with pytest.raises(ValueError):
            s.update_host(np.zeros(5), 1)
        with pytest.raises(hg.HgpuError):
            s.update_host(random_state(cfg), 0)
    finally:
        s.close()
