"""Self-gravity with a live potential on the GPU against the oracle (bit for bit).

useGravity: the potential starts as -density, is relaxed 100 x gaussSeidelMaxIter times
at reset (red-black order, the oracle's and the GPU's schedule of the reference's
in-place relaxation), gaussSeidelMaxIter more times in every callback of the
self-gravity pass, and its gradient drives calcGravityDeriv; the flux kernels subtract
it from the internal energy.  A static potential channel (no useGravity) goes through
the same kernels without the relaxation."""
import itertools

import numpy as np
import pytest

from _cases import SMALL, describe_diff, random_state, same
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu

BOUNDARY = [("PERIODIC", "PERIODIC"), ("MIRROR", "FREEFLOW"), ("FREEFLOW", "MIRROR")]


def compare(hg, oracle_mod, cfg, init, steps, potential=None):
    s = hg.Solver(cfg)
    o = oracle_mod.Oracle(cfg)
    try:
        s.resetState(init, potential)
        o.set_state(init, potential)
        a, b = s.getState(), o.get_state()
        assert same(a, b), "after reset: %s" % describe_diff(a, b)
        assert same(s.getPotential(), o.get_potential()), "potential after reset"
        for k in range(steps):
            dt, do = s.update(1), o.update(1)
            assert dt == do, "step %d: dt %r vs %r" % (k, dt, do)
            a, b = s.getState(), o.get_state()
            assert same(a, b), "step %d: %s" % (k, describe_diff(a, b))
            assert same(s.getPotential(), o.get_potential()), "step %d: potential" % k
    finally:
        s.close()


CASES = list(itertools.product(["EulerRoe", "EulerHLLC", "EulerHLL"], [1, 2, 3],
                               ["ForwardEuler", "RungeKutta2", "RungeKutta4", "RungeKutta3TVD"], [_abi.FP64, _abi.FP32]))


@pytest.mark.parametrize("solver,dim,integ,prec", CASES)
def test_gravity_matches_oracle(hg, oracle_mod, solver, dim, integ, prec):
    size = SMALL[dim]
    cfg = _abi.make_config(solver=solver, size=size, integrator=integ, precision=prec, use_gravity=True,
                           gauss_seidel_max_iter=3, gravitational_constant=.7, boundary=BOUNDARY, limiter="MinMod")
    init = ic.gravity_blobs(size=size, seed=dim, dtype=np.float32 if prec else np.float64)
    compare(hg, oracle_mod, cfg, init, steps=3)


@pytest.mark.parametrize("limiter", ["Superbee", "VanLeer", "Koren"])
def test_gravity_roe_limiters(hg, oracle_mod, limiter):
    cfg = _abi.make_config(solver="EulerRoe", size=(26, 22), integrator="RungeKutta2Heun", use_gravity=True,
                           gauss_seidel_max_iter=4, gravitational_constant=1.3, boundary="PERIODIC", limiter=limiter)
    compare(hg, oracle_mod, cfg, ic.gravity_blobs(size=(26, 22), seed=5), steps=4)


def test_gravity_gs_iterations_and_constant(hg, oracle_mod):
    """gaussSeidelMaxIter 0 (no relaxation: the -density guess stays) and a constant
    that the %.14g define rounds."""
    for iters, G in [(0, 1.), (7, 1. / 3.)]:
        cfg = _abi.make_config(solver="EulerHLLC", size=(30, 12), integrator="ForwardEuler", use_gravity=True,
                               gauss_seidel_max_iter=iters, gravitational_constant=G, boundary="FREEFLOW")
        compare(hg, oracle_mod, cfg, ic.gravity_blobs(size=(30, 12), seed=6), steps=3)


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC", "EulerHLL"])
@pytest.mark.parametrize("prec", [_abi.FP64, _abi.FP32])
def test_static_potential(hg, oracle_mod, solver, prec):
    cfg = _abi.make_config(solver=solver, size=SMALL[2], integrator="RungeKutta2", boundary="FREEFLOW",
                           precision=prec)
    init = random_state(cfg, seed=4, blocky=False)
    pot = np.random.default_rng(5).uniform(-.2, .2, _abi.config_volume(cfg))
    compare(hg, oracle_mod, cfg, init, steps=3, potential=pot)


def test_potential_toggles_between_resets(hg, oracle_mod):
    """The step graph is rebuilt when a reset turns the potential on or off."""
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[2], integrator="RungeKutta4", boundary="PERIODIC")
    init = random_state(cfg, seed=8, blocky=False)
    pot = np.random.default_rng(9).uniform(-.1, .1, _abi.config_volume(cfg))
    s = hg.Solver(cfg)
    try:
        for p in (None, pot, None, pot):
            o = oracle_mod.Oracle(cfg)
            s.resetState(init, p)
            o.set_state(init, p)
            for _ in range(2):
                assert s.update(1) == o.update(1)
            assert same(s.getState(), o.get_state())
    finally:
        s.close()


def test_gravity_display_and_save(hg, oracle_mod, tmp_path):
    """convertToTex's POTENTIAL and ENERGY_INTERNAL see the live potential; the saved
    potential channel is the potential buffer."""
    from test_gpu_output import read_fits
    cfg = _abi.make_config(solver="EulerRoe", size=(20, 18), integrator="RungeKutta2", use_gravity=True,
                           gauss_seidel_max_iter=3, boundary="PERIODIC")
    init = ic.gravity_blobs(size=(20, 18), seed=2)
    s = hg.Solver(cfg)
    o = oracle_mod.Oracle(cfg)
    try:
        s.resetState(init)
        o.set_state(init)
        s.update(2)
        o.update(2)
        names = _abi.display_names(2)
        for name in ("POTENTIAL", "ENERGY_INTERNAL", "PRESSURE"):
            m = names.index(name)
            a, b = s.display(m).reshape(-1), o.display(m).reshape(-1)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name
        idx = s.save(str(tmp_path))
        _, pot = read_fits(str(tmp_path / ("potential%d.fits" % idx)))
        assert np.array_equal(pot.astype(np.float32).reshape(-1), s.getPotential().astype(np.float32))
        assert np.abs(pot).max() > 0
    finally:
        s.close()


def test_adjoint_refuses_live_potential(hg):
    cfg = _abi.make_config(solver="EulerRoe", size=(20, 20), integrator="RungeKutta2", use_gravity=True,
                           gauss_seidel_max_iter=2, boundary="PERIODIC")
    s = hg.Solver(cfg)
    try:
        s.resetState(ic.gravity_blobs(size=(20, 20), seed=1))
        with pytest.raises(hg.HgpuError):
            s.update_frozen_dt([1e-3])
    finally:
        s.close()


def test_gravity_large_grid_finite_and_symmetric(hg):
    """A 256^2 periodic run: the relaxation and source stay finite, a single centred
    blob keeps the x <-> y symmetry of its initial state (the red-black order maps to
    itself under that swap; mirror images of a cell can have the other colour), and the
    potential well sits at the blob."""
    n = 260
    cfg = _abi.make_config(solver="EulerHLLC", size=(n, n), integrator="RungeKutta2", use_gravity=True,
                           gauss_seidel_max_iter=20, boundary="PERIODIC")
    x, y, _ = ic.mesh((n, n), (-.5, -.5, -.5), (.5, .5, .5))
    rho = 1. + 2. * np.exp(-(x * x + y * y) / (2 * .08 ** 2))
    init = ic.build_state_euler(2, 1.4, rho, 0., 0., 0., 10.)
    s = hg.Solver(cfg)
    try:
        s.resetState(init)
        s.update(5)
        st = s.getState().reshape(n, n, 4)
        assert np.isfinite(st).all()
        rho = st[..., 0]
        assert np.allclose(rho, rho.T, rtol=0, atol=1e-9 * rho.max())
        pot = s.getPotential().reshape(n, n)
        inner = pot[2:n - 2, 2:n - 2]
        iy, ix = np.unravel_index(np.argmin(inner), inner.shape)
        assert abs(iy + 2 - (n - 1) / 2) <= 1 and abs(ix + 2 - (n - 1) / 2) <= 1
    finally:
        s.close()
