"""The fused per-direction Runge-Kutta stage (hgpu_set_fused_stages, kernels/roe_fused.cu)
against the default four kernels per stage and the oracle: the state and dt of every
step bit for bit, over grid shapes that exercise the x pass's row segments (253
cells) and the y pass's strips (32 columns x 128 rows, 8-row steps), every boundary
method, REF and SEAM, several tableaus and limiters (compile-time and run-time
dispatched), fixed dt, and the 2048^2 benchmark grid."""
import numpy as np
import pytest

from _cases import describe_diff, random_state, same
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu


def run(hg, cfg, init, steps, fused):
    s = hg.Solver(cfg)
    try:
        if fused:
            s.set_fused_stages(True)
        s.resetState(init)
        out = []
        for _ in range(steps):
            dt = s.update(1)
            out.append((dt, s.getState().copy()))
        assert s.health() & _abi.HEALTH_COPY_TIMEOUT == 0
        return out, s.kernels_per_step()
    finally:
        s.close()


def check(hg, cfg, init, steps=3):
    a, ka = run(hg, cfg, init, steps, False)
    b, kb = run(hg, cfg, init, steps, True)
    for k, ((da, sa), (db, sb)) in enumerate(zip(a, b)):
        assert da == db, "step %d: dt %r (fused %r)" % (k, da, db)
        assert same(sa, sb), "step %d: %s" % (k, describe_diff(sb, sa))
    return ka, kb


SHAPES = [(40, 36), (64, 64), (100, 75), (300, 260), (37, 300), (260, 9), (5, 5)]


@pytest.mark.parametrize("size", SHAPES)
@pytest.mark.parametrize("boundary", ["PERIODIC", "MIRROR", "FREEFLOW"])
def test_fused_shapes_and_boundaries(hg, size, boundary):
    cfg = _abi.make_config(solver="EulerRoe", size=size, boundary=boundary, limiter="MinMod",
                           integrator="RungeKutta4")
    init = random_state(cfg, seed=sum(size), blocky=size[0] % 2 == 0)
    ka, kb = check(hg, cfg, init)
    assert kb == ka - 4 * 2                         # 4 stages: 2 kernels instead of 4


@pytest.mark.parametrize("integrator", ["RungeKutta2", "RungeKutta2Heun", "RungeKutta3", "RungeKutta3TVD",
                                        "RungeKutta4TVD", "RungeKutta4NonTVD", "RungeKutta4_3_8thsRule"])
@pytest.mark.parametrize("limiter", ["Superbee", "VanLeer", "Koren", "MonotizedCentral", "DonorCell"])
def test_fused_integrators_limiters(hg, integrator, limiter):
    cfg = _abi.make_config(solver="EulerRoe", size=(70, 90), boundary=[("PERIODIC", "PERIODIC"),
                                                                      ("MIRROR", "FREEFLOW")],
                           limiter=limiter, integrator=integrator)
    check(hg, cfg, random_state(cfg, seed=7, blocky=limiter == "VanLeer"))


@pytest.mark.parametrize("compat", [_abi.COMPAT_REF, _abi.COMPAT_SEAM])
def test_fused_compat_and_fixed_dt(hg, compat):
    cfg = _abi.make_config(solver="EulerRoe", size=(96, 140), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", compat=compat)
    check(hg, cfg, ic.kelvin_helmholtz(size=(96, 140), seed=3).reshape(-1), steps=4)
    cfg.use_fixed_dt = 1
    cfg.fixed_dt = 2e-4
    check(hg, cfg, ic.kelvin_helmholtz(size=(96, 140), seed=4).reshape(-1), steps=2)


def test_fused_against_oracle(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerRoe", size=(72, 300), boundary="FREEFLOW", limiter="Superbee",
                           integrator="RungeKutta2")
    init = ic.configuration(5, size=(72, 300)).reshape(-1)
    s = hg.Solver(cfg)
    s.set_fused_stages(True)
    s.resetState(init)
    ref = oracle_mod.Oracle(cfg)
    ref.set_state(init)
    for k in range(4):
        dg, dr = s.update(1), ref.update(1)
        a, b = s.getState(), ref.get_state()
        assert dg == dr, (k, dg, dr)
        assert same(a, b), "step %d: %s" % (k, describe_diff(a, b))
    s.close()


def test_fused_kh_2048(hg):
    size = (2048, 2048)
    cfg = _abi.make_config(solver="EulerRoe", size=size, boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", cfl=.5)
    check(hg, cfg, ic.kelvin_helmholtz(size=size, seed=0).reshape(-1), steps=2)


def test_fused_update_host_matches(hg):
    size = (160, 200)
    cfg = _abi.make_config(solver="EulerRoe", size=size, boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4")
    init = ic.kelvin_helmholtz(size=size, seed=6).reshape(-1)
    s = hg.Solver(cfg)
    s.set_fused_stages(True)
    s.resetState(init)
    s.update(2)
    want = s.getState().copy()
    s.set_fused_stages(False)
    s.resetState(init)
    s.update(2)
    assert same(s.getState(), want)
    s.set_fused_stages(True)
    out = np.empty_like(init)
    got, _ = s.update_host(init, 2, out=out)
    assert same(got, want), describe_diff(got, want)
    s.close()


@pytest.mark.parametrize("kw", [dict(integrator="ForwardEuler"), dict(precision=_abi.FP32),
                                dict(size=(64,)), dict(size=(12, 12, 12)), dict(solver="EulerHLLC"),
                                dict(solver="EulerHLL")])
def test_fused_refused(hg, kw):
    base = dict(solver="EulerRoe", size=(40, 36), boundary="PERIODIC", integrator="RungeKutta2")
    base.update(kw)
    s = hg.Solver(_abi.make_config(**base))
    with pytest.raises(hg.HgpuError) as e:
        s.set_fused_stages(True)
    assert e.value.status == _abi.ERR_UNSUPPORTED
    s.set_fused_stages(False)
    s.close()
