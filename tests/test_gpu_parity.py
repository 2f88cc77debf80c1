"""CUDA path vs the CPU oracle, through the C ABI, on the same seeded inputs.

FP64 is required to be bit-identical (sign of zero aside, NaN == NaN), state and
dt, step by step.  FP32 is held to 1e-5 normwise relative difference against the
FP32 oracle after the stated number of steps."""
import itertools

import numpy as np
import pytest

from _cases import SMALL, describe_diff, normwise_rel, random_state, same
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


def run_pair(hg, oracle_mod, cfg, init, steps, exact=True):
    gpu = hg.Solver(cfg)
    ref = oracle_mod.Oracle(cfg)
    gpu.resetState(init)
    ref.set_state(init)
    try:
        for k in range(steps):
            dg = gpu.update(1)
            dr = ref.update(1)
            a, b = gpu.getState(), ref.get_state()
            if exact:
                assert dg == dr, "step %d: dt %r vs oracle %r" % (k, dg, dr)
                assert same(a, b), "step %d: %s" % (k, describe_diff(a, b))
        if not exact:
            return normwise_rel(a, b, gpu.num_states), abs(dg - dr) / abs(dr)
    finally:
        gpu.close()
    return 0.0, 0.0


BOUNDARIES = ["PERIODIC", "MIRROR", "FREEFLOW"]


@pytest.mark.parametrize("dim,bnd", list(itertools.product([1, 2, 3], BOUNDARIES)))
@pytest.mark.parametrize("integrator", _abi.INTEGRATORS)
def test_roe_integrators_boundaries(hg, oracle_mod, dim, bnd, integrator):
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[dim], boundary=bnd, limiter="Superbee",
                           integrator=integrator)
    run_pair(hg, oracle_mod, cfg, random_state(cfg, seed=dim, blocky=True), steps=3)


@pytest.mark.parametrize("limiter", _abi.LIMITERS)
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_roe_limiters(hg, oracle_mod, limiter, dim):
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[dim], boundary="PERIODIC", limiter=limiter,
                           integrator="RungeKutta2")
    # smooth random states keep every limiter finite over several steps
    run_pair(hg, oracle_mod, cfg, random_state(cfg, seed=11), steps=3)


@pytest.mark.parametrize("limiter", _abi.LIMITERS)
def test_roe_limiters_degenerate_ratios(hg, oracle_mod, limiter):
    # blocky states hit r = x/0 and 0/0; VanLeer/CHARM then produce NaN exactly as the reference
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[2], boundary="FREEFLOW", limiter=limiter,
                           integrator="ForwardEuler")
    run_pair(hg, oracle_mod, cfg, random_state(cfg, seed=5, blocky=True), steps=1)


@pytest.mark.parametrize("dim,bnd", list(itertools.product([1, 2, 3], BOUNDARIES)))
@pytest.mark.parametrize("integrator", ["ForwardEuler", "RungeKutta2", "RungeKutta4", "RungeKutta2TVD",
                                        "RungeKutta3TVD", "RungeKutta4TVD"])
def test_hllc(hg, oracle_mod, dim, bnd, integrator):
    cfg = _abi.make_config(solver="EulerHLLC", size=SMALL[dim], boundary=bnd, limiter="VanLeer",
                           integrator=integrator)
    run_pair(hg, oracle_mod, cfg, random_state(cfg, seed=7 + dim, blocky=(dim == 2)), steps=3)


def test_roe_fixed_dt_keeps_stale_basis(hg, oracle_mod):
    # useFixedDT skips Roe::calcTimestep, so the eigenbasis is never computed (Solver.cpp:528)
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[2], boundary="PERIODIC", integrator="RungeKutta2",
                           use_fixed_dt=True, fixed_dt=1e-3)
    run_pair(hg, oracle_mod, cfg, random_state(cfg, seed=1), steps=2)


def test_hllc_fixed_dt(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerHLLC", size=SMALL[2], boundary="PERIODIC", integrator="RungeKutta2",
                           use_fixed_dt=True, fixed_dt=1e-3)
    run_pair(hg, oracle_mod, cfg, random_state(cfg, seed=1), steps=2)


def test_sod_1d(hg, oracle_mod):
    # benchmark config 1 (Sod, superbee, forward Euler, CFL .5, free flow), 200 steps at full size
    cfg = _abi.make_config(solver="EulerRoe", size=(1024,), xmin=(0.,), xmax=(1.,), boundary="FREEFLOW",
                           limiter="Superbee", integrator="ForwardEuler", cfl=.5)
    run_pair(hg, oracle_mod, cfg, ic.sod(size=(1024,)).reshape(-1), steps=200)


def test_kh_roe_small(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerRoe", size=(64, 64), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", cfl=.5)
    run_pair(hg, oracle_mod, cfg, ic.kelvin_helmholtz(size=(64, 64), seed=0).reshape(-1), steps=10)


def test_kh_hllc_small(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerHLLC", size=(64, 64), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", cfl=.5)
    run_pair(hg, oracle_mod, cfg, ic.kelvin_helmholtz(size=(64, 64), seed=0).reshape(-1), steps=10)


def test_grf_hllc_3d_small(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerHLLC", size=(24, 24, 24), xmin=(0, 0, 0), xmax=(1, 1, 1), gamma=5. / 3.,
                           boundary="MIRROR", limiter="VanLeer", integrator="RungeKutta2TVD", cfl=.4)
    init = ic.lognormal_grf(size=(24, 24, 24), corr_cells=4.0, seed=1).reshape(-1)
    run_pair(hg, oracle_mod, cfg, init, steps=5)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6])
def test_quadrant_configurations(hg, oracle_mod, n):
    cfg = _abi.make_config(solver="EulerRoe", size=(32, 32), boundary="FREEFLOW", limiter="Superbee",
                           integrator="RungeKutta2", cfl=.475)
    run_pair(hg, oracle_mod, cfg, ic.configuration(n, size=(32, 32)).reshape(-1), steps=4)


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC"])
def test_fp32_against_fp32_oracle(hg, oracle_mod, solver):
    cfg = _abi.make_config(solver=solver, size=(48, 48), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", precision=_abi.FP32)
    init = ic.kelvin_helmholtz(size=(48, 48), seed=2, dtype=np.float32).reshape(-1)
    err, dterr = run_pair(hg, oracle_mod, cfg, init, steps=100, exact=False)
    assert err <= FP32_TOL, "FP32 normwise relative difference %g after 100 steps" % err


def test_graph_and_plain_launches_agree(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerRoe", size=(40, 36), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4")
    init = random_state(cfg, seed=9)
    a = hg.Solver(cfg)
    b = hg.Solver(cfg)
    b.set_graphs(False)
    a.resetState(init)
    b.resetState(init)
    a.update(4)
    b.update(4)
    assert same(a.getState(), b.getState())
    assert a.kernels_per_step() == b.kernels_per_step() > 0
    a.close()
    b.close()


def test_multi_step_call_matches_single_steps(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerHLLC", size=(30, 30), boundary="FREEFLOW", integrator="RungeKutta2")
    init = random_state(cfg, seed=4)
    a = hg.Solver(cfg)
    b = hg.Solver(cfg)
    a.resetState(init)
    b.resetState(init)
    a.update(5)
    for _ in range(5):
        b.update(1)
    assert same(a.getState(), b.getState())
    assert a.last_dt() == b.last_dt()
    a.close()
    b.close()


def test_step_aliases_match_update(hg):
    """hgpu_step / hgpu_batch_step are hgpu_update / hgpu_batch_update."""
    import ctypes
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[2], boundary="PERIODIC", limiter="Superbee",
                           integrator="RungeKutta2")
    init = random_state(cfg, seed=8)
    a, b = hg.Solver(cfg), hg.Solver(cfg)
    a.resetState(init)
    b.resetState(init)
    a.update(3)
    dt = ctypes.c_double()
    hg.check(hg.lib().hgpu_step(b.h, 3, ctypes.byref(dt)))
    assert same(a.getState(), b.getState()) and dt.value == a.last_dt()
    ba, bb = hg.Batch([cfg, cfg]), hg.Batch([cfg, cfg])
    for bt in (ba, bb):
        bt.set_state(0, init)
        bt.set_state(1, init)
    ba.update(2)
    hg.check(hg.lib().hgpu_batch_step(bb.h, 2))
    assert same(ba.get_state(1), bb.get_state(1))
    for x in (a, b, ba, bb):
        x.close()


@pytest.mark.parametrize("dim,bnd", list(itertools.product([1, 2, 3], BOUNDARIES)))
@pytest.mark.parametrize("integrator", ["ForwardEuler", "RungeKutta2", "RungeKutta4", "RungeKutta3TVD",
                                        "RungeKutta4TVD"])
def test_hll_integrators_boundaries(hg, oracle_mod, dim, bnd, integrator):
    """EulerHLL (res/EulerHLL.cl): Davis-bounded wave speeds, two-state HLL flux."""
    cfg = _abi.make_config(solver="EulerHLL", size=SMALL[dim], boundary=bnd, integrator=integrator)
    run_pair(hg, oracle_mod, cfg, random_state(cfg, seed=20 + dim, blocky=True), steps=3)


def test_hll_kh_and_quadrants(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerHLL", size=(64, 64), boundary="PERIODIC", integrator="RungeKutta4")
    run_pair(hg, oracle_mod, cfg, ic.kelvin_helmholtz(size=(64, 64), seed=2).reshape(-1), steps=10)
    for n in (1, 3, 6):
        cfg = _abi.make_config(solver="EulerHLL", size=(32, 32), boundary="FREEFLOW", integrator="RungeKutta2",
                               cfl=.475)
        run_pair(hg, oracle_mod, cfg, ic.configuration(n, size=(32, 32)).reshape(-1), steps=6)


def test_hll_fp32(hg, oracle_mod):
    cfg = _abi.make_config(solver="EulerHLL", size=(48, 40), boundary="PERIODIC", integrator="RungeKutta2",
                           precision=_abi.FP32)
    err, dterr = run_pair(hg, oracle_mod, cfg, random_state(cfg, seed=4), steps=100, exact=False)
    assert err <= FP32_TOL and dterr <= FP32_TOL, (err, dterr)
