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
