"""Host-side configuration rules restated from the reference (no GPU needed)."""
import numpy as np
import pytest

from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic


def test_dx_baked_to_six_significant_digits(oracle_mod):
    # toNumericString<double> (include/HydroGPU/toNumericString.h:12-22)
    cfg = _abi.make_config(size=(2048, 2048))
    dim, dx, gamma, _ = oracle_mod.resolve(cfg)
    assert dim == 2 and dx[0] == 0.000488281 and dx[1] == 0.000488281
    cfg = _abi.make_config(size=(1024,), xmin=(0.,), xmax=(1.,))
    assert oracle_mod.resolve(cfg)[1][0] == 0.000976562
    cfg = _abi.make_config(size=(256, 256, 256), xmin=(0, 0, 0), xmax=(1, 1, 1))
    assert oracle_mod.resolve(cfg)[1] == [0.00390625] * 3


def test_gamma_baked_like_lua_numbers(oracle_mod):
    cfg = _abi.make_config(size=(16, 16), gamma=5. / 3.)
    assert oracle_mod.resolve(cfg)[2] == 1.6666666666667
    cfg = _abi.make_config(size=(16, 16), gamma=7. / 5.)
    assert oracle_mod.resolve(cfg)[2] == 1.4


def test_seam_mode_keeps_exact_constants(oracle_mod):
    cfg = _abi.make_config(size=(2048, 2048), compat=_abi.COMPAT_SEAM, gamma=5. / 3.)
    dim, dx, gamma, _ = oracle_mod.resolve(cfg)
    assert dx[0] == 1.0 / 2048 and gamma == 5. / 3.


def test_dim_is_last_axis_with_size_above_one(oracle_mod):
    assert oracle_mod.resolve(_abi.make_config(size=(32,)))[0] == 1
    assert oracle_mod.resolve(_abi.make_config(size=(32, 8)))[0] == 2
    assert oracle_mod.resolve(_abi.make_config(size=(8, 8, 8)))[0] == 3


@pytest.mark.parametrize("kw", [dict(size=(4, 16)), dict(size=(16, 16), limiter=99), dict(size=(16, 16), integrator=-1),
                                dict(size=(16, 16), xmin=(1, 1), xmax=(0, 0))])
def test_invalid_configs_rejected(oracle_mod, kw):
    with pytest.raises(ValueError):
        oracle_mod.resolve(_abi.make_config(**kw))


def test_name_registries_match_reference_keys():
    with pytest.raises(ValueError):
        _abi.make_config(limiter="NoSuchLimiter")
    cfg = _abi.make_config(solver="EulerHLLC", limiter="MinMod", integrator="RungeKutta4TVD",
                           boundary=[{"min": "PERIODIC", "max": "MIRROR"}, ("FREEFLOW", "NONE")])
    assert cfg.solver == 1 and cfg.limiter == 8 and cfg.integrator == 10
    assert list(cfg.boundary[0]) == [0, 1] and list(cfg.boundary[1]) == [2, -1]


def test_build_state_euler_energy():
    # E = rho * (.5 |v|^2 + p / ((gamma - 1) rho))  (res/util.lua:36-80)
    st = ic.build_state_euler(2, 1.4, np.array([2.0]), np.array([.5]), np.array([-.25]), 0.0, np.array([2.5]))
    rho, mx, my, e = st[0]
    assert rho == 2.0 and mx == 1.0 and my == -.5
    assert e == 2.0 * (.5 * (.25 + .0625 + 0.0) + 2.5 / ((1.4 - 1) * 2.0))


def test_initial_conditions_shapes_and_ranges():
    kh = ic.kelvin_helmholtz(size=(64, 32), seed=0)
    assert kh.shape == (1, 32, 64, 4)
    assert set(np.unique(kh[..., 0])) == {1.0, 2.0}
    sod = ic.sod(size=(100,))
    assert sod.shape == (1, 1, 100, 3) and sod[0, 0, 0, 0] == 1.0 and sod[0, 0, -1, 0] == .125
    q = ic.configuration(1, size=(8, 8))
    assert q[0, 7, 7, 0] == 1.0 and q[0, 0, 0, 0] == .1072
    g = ic.lognormal_grf(size=(16, 16, 16), corr_cells=3.0)
    assert abs(g[..., 0].mean() - 1.0) < 1e-12 and np.all(g[..., 0] > 0)
    probs = ic.random_quadrant_problems(64, seed=2)
    sides = [p["side"] for p in probs]
    assert min(sides) >= 32 and max(sides) <= 512 and all(s % 16 == 0 for s in sides)


def test_display_names():
    assert _abi.display_names(1) == ["DENSITY", "VELOCITY", "VELOCITY_X", "PRESSURE", "ENERGY_INTERNAL",
                                     "ENERGY_KINETIC", "ENERGY_TOTAL", "POTENTIAL"]
    assert len(_abi.display_names(3)) == 10
    assert _abi.display_index(2, "pressure") == 4
    with pytest.raises(ValueError):
        _abi.display_index(1, "VELOCITY_Y")
