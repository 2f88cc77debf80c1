"""Batched problems (hgpu_batch_*) against the same problems run alone.

A batch advances many independent problems of uneven sizes in persistent launches;
each problem must come out bit-identical (FP64 and FP32 alike: the per-cell
arithmetic is the single-problem code) to an hgpu_update run of that problem, state
and dt, for every tuning the autotuner may pick.  A few problems are also checked
against the oracle directly."""
import os

import numpy as np
import pytest

from _cases import describe_diff, random_state, same
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu

BOUNDS = ["PERIODIC", "MIRROR", "FREEFLOW"]


def mixed_configs(solver, dim, integrator, limiter, n, seed, precision=_abi.FP64):
    """n problems of one solver/dim/integrator/limiter with their own sizes, domains,
    gamma, cfl and per-side boundary methods."""
    rng = np.random.default_rng(seed)
    lo, hi = {1: (8, 70), 2: (8, 30), 3: (7, 13)}[dim]
    cfgs = []
    for k in range(n):
        size = tuple(int(rng.integers(lo, hi)) for _ in range(dim))
        bnd = [(BOUNDS[int(rng.integers(3))], BOUNDS[int(rng.integers(3))]) for _ in range(dim)]
        xmin = tuple(float(rng.uniform(-1, 0)) for _ in range(dim))
        xmax = tuple(a + float(rng.uniform(.5, 2)) for a in xmin)
        cfgs.append(_abi.make_config(solver=solver, size=size, xmin=xmin, xmax=xmax,
                                     gamma=[1.4, 5. / 3.][k % 2], cfl=[.5, .3, .8][k % 3], boundary=bnd,
                                     limiter=limiter, integrator=integrator, precision=precision))
    return cfgs


def run_alone(hg, cfg, init, steps):
    s = hg.Solver(cfg)
    try:
        s.resetState(init)
        out, dts = [], []
        for _ in range(steps):
            dts.append(s.update(1))
            out.append(s.getState().copy())
        return out, dts
    finally:
        s.close()


def check_batch(hg, cfgs, steps=3, tunings=(None,), seed=5, blocky=True):
    inits = [random_state(c, seed=seed + k, blocky=blocky and k % 2 == 0) for k, c in enumerate(cfgs)]
    alone = [run_alone(hg, c, x, steps) for c, x in zip(cfgs, inits)]
    for tu in tunings:
        b = hg.Batch(cfgs)
        try:
            if tu is not None:
                b.set_tuning(*tu)
            for p, x in enumerate(inits):
                b.set_state(p, x)
            for k in range(steps):
                b.update(1)
                dts = b.dts()
                for p in range(len(cfgs)):
                    a = b.get_state(p)
                    ref, rdt = alone[p][0][k], alone[p][1][k]
                    assert dts[p] == rdt, "tuning %r problem %d step %d: dt %r vs %r" % (tu, p, k, dts[p], rdt)
                    assert same(a, ref), "tuning %r problem %d step %d: %s" % (tu, p, k, describe_diff(a, ref))
        finally:
            b.close()


@pytest.mark.parametrize("integrator", ["ForwardEuler", "RungeKutta2", "RungeKutta4", "RungeKutta3TVD",
                                        "RungeKutta2Heun"])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_roe_batch_matches_alone(hg, dim, integrator):
    check_batch(hg, mixed_configs("EulerRoe", dim, integrator, "Superbee", n=7, seed=dim))


@pytest.mark.parametrize("integrator", ["ForwardEuler", "RungeKutta2TVD", "RungeKutta4"])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_hllc_batch_matches_alone(hg, dim, integrator):
    check_batch(hg, mixed_configs("EulerHLLC", dim, integrator, "Superbee", n=6, seed=10 + dim), blocky=False)


@pytest.mark.parametrize("integrator", ["ForwardEuler", "RungeKutta2", "RungeKutta4"])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_hll_batch_matches_alone(hg, dim, integrator):
    check_batch(hg, mixed_configs("EulerHLL", dim, integrator, "Superbee", n=6, seed=50 + dim), blocky=False)


@pytest.mark.parametrize("limiter", ["MinMod", "VanLeer", "MonotizedCentral", "DonorCell", "LaxWendroff"])
def test_roe_batch_limiters(hg, limiter):
    check_batch(hg, mixed_configs("EulerRoe", 2, "RungeKutta2", limiter, n=4, seed=3), steps=2, blocky=False)


@pytest.mark.parametrize("dim,tunings", [
    (1, [((256, 1, 1), 1, 0), ((128, 1, 1), 0, 2), ((7, 1, 1), 1, 1), ((512, 1, 1), 0, 0, 1, 2),
         ((256, 1, 1), 1, 0, 0, 1), ((256, 1, 1), 0, -1, 1, 1)]),
    (2, [((32, 8, 1), 1, 0), ((16, 16, 1), 0, 0), ((64, 4, 1), 1, 2), ((5, 3, 1), 1, 1), ((16, 8, 1), 0, 1),
         ((32, 8, 1), 1, 0, 0, 1), ((32, 16, 1), 0, 0, 1, 2), ((32, 32, 1), 0, 2, 0, 4), ((7, 9, 1), 0, 0, 1, 3),
         ((16, 16, 1), 1, -1, 1, 1), ((32, 16, 1), 0, -1, 0, 2)]),
    (3, [((32, 4, 2), 1, 0), ((8, 8, 4), 0, 2), ((3, 5, 2), 1, 1), ((32, 4, 4), 0, 0, 1, 2),
         ((32, 4, 2), 1, 0, 0, 1), ((32, 4, 2), 1, -1, 1, 1)]),
])
def test_batch_tuning_invariant(hg, dim, tunings):
    """Every tile shape, staging choice, persistent grid, flux form (one or two passes)
    and number of cells per thread gives the same bits."""
    check_batch(hg, mixed_configs("EulerRoe", dim, "RungeKutta4", "MinMod", n=5, seed=20 + dim), steps=2,
                tunings=tunings)


def test_batch_fixed_dt(hg):
    cfgs = mixed_configs("EulerRoe", 2, "RungeKutta3TVD", "Superbee", n=4, seed=31)
    for c in cfgs:
        c.use_fixed_dt = 1
        c.fixed_dt = .0007
    check_batch(hg, cfgs, steps=2)
    cfgs = mixed_configs("EulerHLLC", 2, "ForwardEuler", "Superbee", n=4, seed=32)
    for c in cfgs:
        c.use_fixed_dt = 1
        c.fixed_dt = .0003
    check_batch(hg, cfgs, steps=2, blocky=False)


def test_batch_fp32(hg):
    check_batch(hg, mixed_configs("EulerRoe", 2, "RungeKutta2", "Superbee", n=5, seed=41, precision=_abi.FP32),
                steps=3)
    check_batch(hg, mixed_configs("EulerHLLC", 2, "RungeKutta4", "Superbee", n=5, seed=42, precision=_abi.FP32),
                steps=3, blocky=False)


def quadrant_sweep(n, seed=2, lo=16, hi=64, integrator="RungeKutta2", limiter="Superbee"):
    cfgs, inits = [], []
    for pr in ic.random_quadrant_problems(n=n, seed=seed, lo=lo, hi=hi):
        cfg = _abi.make_config(solver="EulerRoe", size=(pr["side"], pr["side"]), boundary=pr["boundary"],
                               limiter=limiter, integrator=integrator)
        cfgs.append(cfg)
        inits.append(ic.quadrant((pr["side"], pr["side"]), pr["quadrants"]).reshape(-1))
    return cfgs, inits


def test_quadrant_sweep_vs_oracle(hg, oracle_mod):
    """Random four-quadrant Riemann problems (the batched sweep's inputs, smaller
    sides) against the oracle, problem by problem."""
    cfgs, inits = quadrant_sweep(6)
    b = hg.Batch(cfgs)
    try:
        for p, x in enumerate(inits):
            b.set_state(p, x)
        b.update(2)
        dts = b.dts()
        for p, (c, x) in enumerate(zip(cfgs, inits)):
            o = oracle_mod.Oracle(c)
            o.set_state(x)
            o.update(1)
            dt = o.update(1)
            a, ref = b.get_state(p), o.get_state()
            assert dts[p] == dt
            assert same(a, ref), "problem %d: %s" % (p, describe_diff(a, ref))
    finally:
        b.close()


def test_batch_autotune_cache(hg, tmp_path):
    cfgs, inits = quadrant_sweep(12, lo=16, hi=96)
    cache = str(tmp_path / "tune.txt")
    b = hg.Batch(cfgs)
    try:
        for p, x in enumerate(inits):
            b.set_state(p, x)
        before = [b.get_state(p) for p in range(len(cfgs))]
        tu = b.autotune(cache, steps=1)
        after = [b.get_state(p) for p in range(len(cfgs))]
        assert all(same(x, y) for x, y in zip(before, after)), "autotune must restore the state"
        b.update(2)
        res = [b.get_state(p) for p in range(len(cfgs))]
    finally:
        b.close()
    lines = open(cache).read().split("\n")
    assert lines[0].startswith("v2-roe-2d-")
    b2 = hg.Batch(cfgs)
    try:
        assert b2.autotune(cache, steps=1) == tu          # looked up, not re-timed
        assert open(cache).read().count("\n") == 1
        for p, x in enumerate(inits):
            b2.set_state(p, x)
        b2.update(2)
        for p in range(len(cfgs)):
            assert same(b2.get_state(p), res[p])
    finally:
        b2.close()


def test_batch_info_and_health(hg):
    cfgs, inits = quadrant_sweep(5)
    b = hg.Batch(cfgs)
    try:
        for p, x in enumerate(inits):
            b.set_state(p, x)
        b.update(1)
        n, cells, k = b.info()
        assert n == 5
        assert cells >= sum(c.size[0] * c.size[1] for c in cfgs)
        # boundary, basis, dt, finalize; RK2: 2 x (dq, flux corrections, flux transforms, combine); state check
        assert k == 1 + 2 + 1 + 2 * 4 + 1
        assert b.health() == 0
        with pytest.raises(hg.HgpuError):
            b.set_state(5, inits[0])
        with pytest.raises(hg.HgpuError):
            b.set_state(0, inits[1][:-4])
    finally:
        b.close()
