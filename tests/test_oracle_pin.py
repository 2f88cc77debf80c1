"""The oracle restatement against the reference's own kernels ("refcl").

refcl is HydroGPU's res/*.cl compiled for the CPU (oracle/refcl/build_refcl.py);
it exists only where oracle/_ref/ was built.  Every case must agree bit for bit,
state and dt, step by step."""
import itertools

import numpy as np
import pytest

from _cases import SMALL, describe_diff, random_state, same
from hydrodynamicsgpu_gb300 import _abi


@pytest.fixture(scope="module")
def refcl(oracle_mod):
    if not oracle_mod.refcl_available():
        try:
            oracle_mod.build_refcl(quiet=True)
        except Exception as e:  # pragma: no cover
            pytest.skip("refcl not buildable here: %s" % e)
    if not oracle_mod.refcl_available():
        pytest.skip("refcl not built")
    return oracle_mod


def pin(mod, cfg, init, steps):
    o = mod.Oracle(cfg)
    r = mod.Refcl(cfg)
    o.set_state(init)
    r.set_state(init)
    for k in range(steps):
        do, dr = o.update(1), r.update(1)
        a, b = o.get_state(), r.get_state()
        assert do == dr, "step %d dt %r vs %r" % (k, do, dr)
        assert same(a, b), "step %d: %s" % (k, describe_diff(a, b))


CASES = []
for solver, dim, integ, bnd, prec in itertools.product(
        ["EulerRoe", "EulerHLLC", "EulerHLL"], [1, 2, 3], _abi.INTEGRATORS, ["PERIODIC", "MIRROR", "FREEFLOW"], [0, 1]):
    CASES.append((solver, dim, integ, bnd, prec))


@pytest.mark.parametrize("solver,dim,integ,bnd,prec", CASES[::3])
def test_pin_integrators_boundaries(refcl, solver, dim, integ, bnd, prec):
    cfg = _abi.make_config(solver=solver, size=SMALL[dim], boundary=bnd, limiter="Superbee", integrator=integ,
                           precision=prec)
    pin(refcl, cfg, random_state(cfg, seed=dim + prec, blocky=True), steps=2)


@pytest.mark.parametrize("limiter", _abi.LIMITERS)
@pytest.mark.parametrize("blocky", [False, True])
def test_pin_limiters(refcl, limiter, blocky):
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[2], boundary="PERIODIC", limiter=limiter,
                           integrator="RungeKutta2")
    pin(refcl, cfg, random_state(cfg, seed=3, blocky=blocky), steps=1 if blocky else 3)


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC", "EulerHLL"])
def test_pin_fixed_dt(refcl, solver):
    cfg = _abi.make_config(solver=solver, size=SMALL[2], boundary="FREEFLOW", integrator="RungeKutta4",
                           use_fixed_dt=True, fixed_dt=2e-3)
    pin(refcl, cfg, random_state(cfg, seed=8), steps=2)


def test_pin_gamma_five_thirds(refcl):
    cfg = _abi.make_config(solver="EulerHLLC", size=(9, 8, 7), xmin=(0, 0, 0), xmax=(1, 1, 1), gamma=5. / 3.,
                           boundary="MIRROR", integrator="RungeKutta2TVD", cfl=.4)
    pin(refcl, cfg, random_state(cfg, seed=2), steps=3)


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC", "EulerHLL"])
@pytest.mark.parametrize("dim,prec", [(1, 0), (2, 0), (3, 0), (2, 1), (3, 1)])
def test_pin_display(refcl, solver, dim, prec):
    """The display scalar (convertToTex, res/EulerMHDCommon.cl:4-116) restated in the
    oracle against the reference's own kernel, every display method."""
    cfg = _abi.make_config(solver=solver, size=SMALL[dim], boundary="PERIODIC", integrator="RungeKutta2",
                           precision=prec)
    init = random_state(cfg, seed=dim + 9)
    o, r = refcl.Oracle(cfg), refcl.Refcl(cfg)
    o.set_state(init)
    r.set_state(init)
    o.update(1)
    r.update(1)
    for m in range(len(_abi.display_names(dim))):
        assert np.array_equal(o.display(m), r.display(m), equal_nan=True), m


# ---------------- self-gravity (useGravity) and the static potential channel ----------------
def pin_gravity(mod, cfg, init, steps, potential=None):
    o = mod.Oracle(cfg)
    r = mod.Refcl(cfg)
    o.set_state(init, potential)
    r.set_state(init, potential)
    assert same(o.get_state(), r.get_state()), "after reset"
    assert same(o.get_potential(), r.get_potential()), "potential after reset"
    for k in range(steps):
        do, dr = o.update(1), r.update(1)
        assert do == dr, "step %d dt %r vs %r" % (k, do, dr)
        a, b = o.get_state(), r.get_state()
        assert same(a, b), "step %d: %s" % (k, describe_diff(a, b))
        assert same(o.get_potential(), r.get_potential()), "step %d potential" % k


GRAVITY_CASES = list(itertools.product(["EulerRoe", "EulerHLLC", "EulerHLL"], [1, 2, 3],
                                       ["ForwardEuler", "RungeKutta2Heun", "RungeKutta4", "RungeKutta3TVD"], [0, 1]))


@pytest.mark.parametrize("solver,dim,integ,prec", GRAVITY_CASES[::2])
def test_pin_gravity(refcl, solver, dim, integ, prec):
    """useGravity: -density start, 100 x maxIter relaxations at reset, maxIter per
    callback, calcGravityDeriv; mixed boundaries (MIRROR's potential ghosts are free flow)."""
    from hydrodynamicsgpu_gb300 import initconds as ic
    size = SMALL[dim]
    cfg = _abi.make_config(solver=solver, size=size, integrator=integ, precision=prec, use_gravity=True,
                           gauss_seidel_max_iter=3, gravitational_constant=.7,
                           boundary=[("PERIODIC", "PERIODIC"), ("MIRROR", "FREEFLOW"), ("FREEFLOW", "MIRROR")])
    init = ic.gravity_blobs(size=size, seed=dim + 10 * prec, dtype=np.float32 if prec else np.float64)
    pin_gravity(refcl, cfg, init, steps=2)


@pytest.mark.parametrize("solver", ["EulerRoe", "EulerHLLC", "EulerHLL"])
def test_pin_static_potential(refcl, solver):
    """No useGravity, a nonzero potential channel: the flux kernels and the source
    term see it, and the reset adds it to the total energy."""
    cfg = _abi.make_config(solver=solver, size=SMALL[2], integrator="RungeKutta2", boundary="FREEFLOW")
    init = random_state(cfg, seed=4, blocky=False)
    pot = np.random.default_rng(5).uniform(-.2, .2, _abi.config_volume(cfg))
    pin_gravity(refcl, cfg, init, steps=3, potential=pot)


def test_relaxation_fixed_point_is_order_independent(oracle_mod):
    """The reference's relaxation launch is an in-place update whose result depends on
    the order of its work-items; the oracle and the GPU use the red-black order.  Every
    order converges to the same discrete Poisson solution: run to convergence, the
    red-black result equals a plain lexicographic Gauss-Seidel (the order a sequential
    device runs) to round-off."""
    from hydrodynamicsgpu_gb300 import initconds as ic
    size = (14, 12)
    cfg = _abi.make_config(solver="EulerRoe", size=size, use_gravity=True, gauss_seidel_max_iter=40,
                           gravitational_constant=1., boundary="FREEFLOW")
    init = ic.gravity_blobs(size=size, seed=3)
    o = oracle_mod.Oracle(cfg)
    o.set_state(init)
    red_black = o.get_potential().reshape(size[1], size[0])
    # lexicographic Gauss-Seidel of gravityPotentialPoissonRelax (res/SelfGravitation.cl:20-63)
    _, dx, _, G = oracle_mod.resolve(cfg)
    rho = init.reshape(size[1], size[0], -1)[..., 0]
    phi = -rho.copy()
    diag = -2. * (1. / (dx[0] * dx[0]) + 1. / (dx[1] * dx[1]))
    for _ in range(4000):
        for y in range(2, size[1] - 2):
            for x in range(2, size[0] - 2):
                s = 0.
                if x < size[0] - 3:
                    s += phi[y, x + 1] / (dx[0] * dx[0])
                if x > 2:
                    s += phi[y, x - 1] / (dx[0] * dx[0])
                if y < size[1] - 3:
                    s += phi[y + 1, x] / (dx[1] * dx[1])
                if y > 2:
                    s += phi[y - 1, x] / (dx[1] * dx[1])
                phi[y, x] = (4. * np.pi * G * rho[y, x] - s) / diag
    inner = (slice(2, size[1] - 2), slice(2, size[0] - 2))
    err = np.abs(red_black[inner] - phi[inner]).max() / np.abs(phi[inner]).max()
    assert err < 1e-12, err
