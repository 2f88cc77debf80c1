"""The benchmark configurations at their full sizes.

Against the oracle, bit for bit (FP64) or within 1e-5 (FP32), for the first steps
of the 2048^2 Kelvin-Helmholtz runs (EulerRoe and EulerHLLC, RK4, MinMod) and the
256^3 log-normal EulerHLLC run (TVD-RK2, VanLeer, mirror), which the oracle finishes
in seconds.  Over more steps, through properties that do not depend on the size:
translation equivariance and conserved totals on the periodic torus (the SEAM
scheme, whose periodic seam faces coincide), the FP32 error against FP64, and the
512-problem batched sweep coming out bit-identical to its problems run alone."""
import math

import numpy as np
import pytest

from _cases import describe_diff, normwise_rel, same
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu

KH = (2048, 2048)
GRF = (256, 256, 256)


def kh_config(solver, **kw):
    return _abi.make_config(solver=solver, size=KH, boundary="PERIODIC", limiter="MinMod",
                            integrator="RungeKutta4", cfl=.5, **kw)


def against_oracle(hg, oracle_mod, cfg, init, steps, exact=True):
    gpu = hg.Solver(cfg)
    ref = oracle_mod.Oracle(cfg)
    try:
        gpu.resetState(init)
        ref.set_state(init)
        for k in range(steps):
            dg, dr = gpu.update(1), ref.update(1)
            a, b = gpu.getState(), ref.get_state()
            if exact:
                assert dg == dr, "step %d: dt %r vs oracle %r" % (k, dg, dr)
                assert same(a, b), "step %d: %s" % (k, describe_diff(a, b))
            else:
                err = normwise_rel(a, b, gpu.num_states)
                assert err <= 1e-5 and abs(dg - dr) <= 1e-5 * abs(dr), (k, err, dg, dr)
    finally:
        gpu.close()


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC"])
def test_kh_2048_fp64_vs_oracle(hg, oracle_mod, solver):
    against_oracle(hg, oracle_mod, kh_config(solver), ic.kelvin_helmholtz(size=KH, seed=0).reshape(-1), steps=2)


def test_kh_2048_fp32_vs_oracle(hg, oracle_mod):
    cfg = kh_config("EulerRoe", precision=_abi.FP32)
    init = ic.kelvin_helmholtz(size=KH, seed=0).astype(np.float32).reshape(-1)
    against_oracle(hg, oracle_mod, cfg, init, steps=2, exact=False)


def test_grf_256cubed_hllc_fp64_vs_oracle(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerHLLC", size=GRF, xmin=(0, 0, 0), xmax=(1, 1, 1), gamma=5. / 3.,
                           boundary="MIRROR", limiter="VanLeer", integrator="RungeKutta2TVD", cfl=.4)
    against_oracle(hg, oracle_mod, cfg, ic.lognormal_grf(size=GRF, seed=1).reshape(-1), steps=1)


def interior(state, n):
    return state.reshape(KH[1], KH[0], n)[2:-2, 2:-2]


def periodic(inner):
    """A full KH-sized state around the interior `inner`, its two ghost layers per
    side the periodic images (what the periodic boundary pass writes)."""
    return np.pad(inner, ((2, 2), (2, 2), (0, 0)), mode="wrap").reshape(-1)


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC"])
def test_kh_2048_translation_equivariance(hg, solver):
    """On the periodic torus every cell runs the same arithmetic on its neighbourhood
    and dt is a minimum over all cells, so a run from the interior rolled by (dy, dx)
    cells is the rolled run, bit for bit, dt included, at every step.  The shifts are
    not multiples of any tile edge."""
    cfg = kh_config(solver, compat=_abi.COMPAT_SEAM)
    u0 = interior(ic.kelvin_helmholtz(size=KH, seed=3).reshape(-1), 4)
    shift = (1029, 517)
    runs = []
    for inner in (u0, np.roll(u0, shift, axis=(0, 1))):
        s = hg.Solver(cfg)
        s.resetState(periodic(inner))
        dts = [s.update(1) for _ in range(25)]
        runs.append((dts, interior(s.getState(), 4)))
        s.close()
    (dta, a), (dtb, b) = runs
    assert dta == dtb
    rolled = np.roll(a, shift, axis=(0, 1))
    assert same(rolled, b), describe_diff(rolled, b)


def exact_totals(state):
    """Interior totals of rho, m_x, m_y, E, each summed exactly (math.fsum: numpy's
    reduction down a strided column accumulates row by row and its own rounding,
    ~1e-13 of the total at 2044^2 cells, would hide the scheme's)."""
    u = interior(state, 4).reshape(-1, 4)
    return np.array([math.fsum(u[:, j]) for j in range(4)]), np.abs(u).sum(0)


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC"])
def test_kh_2048_conserves_totals(hg, solver):
    """Every face flux enters its two cells with opposite signs, so the totals move
    only by the rounding of each cell's state additions: measured at most 2e-16 of
    the total after 50 steps."""
    cfg = kh_config(solver, compat=_abi.COMPAT_SEAM)
    u0 = ic.kelvin_helmholtz(size=KH, seed=4).reshape(-1)
    s = hg.Solver(cfg)
    s.resetState(u0)
    t0, scale = exact_totals(u0)
    s.update(50)
    t1, _ = exact_totals(s.getState())
    s.close()
    drift = np.abs(t1 - t0) / scale
    assert np.all(drift <= 1e-15), drift


def test_kh_2048_fp32_error_against_fp64(hg):
    """KH 2048^2 EulerRoe RK4 after 100 steps, FP32 against FP64 (each with its own
    CFL dt): normwise relative difference per conserved variable below 1e-4."""
    u0 = ic.kelvin_helmholtz(size=KH, seed=0).reshape(-1)
    out = {}
    for prec in (_abi.FP64, _abi.FP32):
        s = hg.Solver(kh_config("EulerRoe", precision=prec))
        s.resetState(u0.astype(np.float32) if prec == _abi.FP32 else u0)
        s.update(100)
        out[prec] = s.getState().astype(np.float64).reshape(-1, 4)
        s.close()
    a, b = out[_abi.FP32], out[_abi.FP64]
    err = np.max(np.abs(a - b), axis=0) / np.max(np.abs(b), axis=0)
    assert np.all(err <= 1e-4), err


def test_batched_sweep_512_matches_alone(hg):
    """The batched workload itself (512 four-quadrant problems, sides 32-512, seed 2,
    EulerRoe RK2 Superbee): after 3 steps every problem's state and each step's dt are
    those of the same problem run alone."""
    cfgs, inits = [], []
    for pr in ic.random_quadrant_problems(n=512, seed=2):
        side = pr["side"]
        cfgs.append(_abi.make_config(solver="EulerRoe", size=(side, side), boundary=pr["boundary"],
                                     limiter="Superbee", integrator="RungeKutta2"))
        inits.append(ic.quadrant((side, side), pr["quadrants"]).reshape(-1))
    steps = 3
    b = hg.Batch(cfgs)
    try:
        for p, x in enumerate(inits):
            b.set_state(p, x)
        dts = []
        for _ in range(steps):
            b.update(1)
            dts.append(np.array(b.dts()))
        finals = [b.get_state(p) for p in range(len(cfgs))]
    finally:
        b.close()
    for p, (c, x) in enumerate(zip(cfgs, inits)):
        s = hg.Solver(c)
        s.resetState(x)
        for k in range(steps):
            d = s.update(1)
            assert d == dts[k][p], "problem %d step %d: dt %r vs batched %r" % (p, k, d, dts[k][p])
        a = s.getState()
        s.close()
        assert same(finals[p], a), "problem %d: %s" % (p, describe_diff(finals[p], a))
