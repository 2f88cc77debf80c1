"""hgpu_config_from_file / hgpu_config_from_string: the reference's config.lua keys
read from a settings file (src/HydroGPUApp.cpp:157-208, :330; src/Solver/Solver.cpp:
196-197, 285-307).  Host-only calls: these run without a GPU."""
import ctypes
import math
import os

import pytest

from hydrodynamicsgpu_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
CONFIGS = os.path.join(HERE, "golden", "config")


def fields(cfg):
    return {name: (list(getattr(cfg, name)) if name in ("size", "xmin", "xmax") else
                   [list(r) for r in cfg.boundary] if name == "boundary" else getattr(cfg, name))
            for name, _ in _abi.HgpuConfig._fields_ if name != "reserved"}


def read(hg, text):
    cfg = _abi.HgpuConfig()
    st = hg.lib().hgpu_config_from_string(text.encode(), ctypes.byref(cfg))
    return st, cfg, hg.lib().hgpu_last_error().decode()


def test_kh_benchmark_file(hg):
    cfg = hg.config_from_file(os.path.join(CONFIGS, "kh2048_roe_rk4.lua"))
    want = _abi.make_config(solver="EulerRoe", size=(2048, 2048), boundary="PERIODIC", limiter="MinMod",
                            integrator="RungeKutta4", cfl=.5)
    assert fields(cfg) == fields(want)


def test_grf_file(hg):
    cfg = hg.config_from_file(os.path.join(CONFIGS, "grf256_hllc_tvdrk2.lua"))
    want = _abi.make_config(solver="EulerHLLC", size=(256, 256, 256), xmin=(0, 0, 0), xmax=(1, 1, 1),
                            gamma=5. / 3., boundary="MIRROR", limiter="VanLeer", integrator="RungeKutta2TVD",
                            cfl=.4, gravitational_constant=.5)
    assert fields(cfg) == fields(want)
    assert cfg.gamma == 5. / 3.           # Lua arithmetic in double; the program bakes it with %.14g


def test_slope_limiter_name_is_not_the_key_the_solver_reads(hg):
    """res/config.lua assigns slopeLimiterName while Solver.cpp:285-287 reads
    slopeLimiter: the shipped config's choice never reaches the solver."""
    cfg = hg.config_from_file(os.path.join(CONFIGS, "sod_limiter_name_quirk.lua"))
    assert cfg.limiter == _abi.LIMITERS.index("Superbee")
    assert list(cfg.size) == [1024, 1, 1] and cfg.xmin[0] == 0 and cfg.xmax[0] == 1
    assert cfg.xmin[1] == -.5 and cfg.xmax[2] == .5   # entries the file leaves out keep the defaults


def test_gravity_fixed_dt_mixed_boundaries(hg):
    cfg = hg.config_from_file(os.path.join(CONFIGS, "blobs_gravity_fixed_dt.lua"))
    assert cfg.solver == _abi.SOLVERS["EulerHLL"]
    assert cfg.integrator == _abi.INTEGRATORS.index("RungeKutta4_3_8thsRule")
    assert list(cfg.size) == [96, 64, 1]
    assert [list(r) for r in cfg.boundary] == [[0, 0], [1, 2], [-1, -1]]
    assert cfg.use_fixed_dt == 1 and cfg.fixed_dt == 2.5e-4
    assert cfg.use_gravity == 1 and cfg.gauss_seidel_max_iter == 16
    assert cfg.gamma == 7 / 5 and cfg.gravitational_constant == 4 * math.pi * 1e-1


def test_cfl_is_a_c_float(hg):
    st, cfg, _ = read(hg, "solverName = 'EulerRoe'\ncfl = 0.4\n")
    assert st == 0 and cfg.cfl == ctypes.c_float(.4).value


@pytest.mark.parametrize("text,expect", [
    ("solverName = 'EulerRoe'\nx = -2^2\n", None),                      # -(2^2) as in Lua
    ("solverName = 'EulerRoe'\nsize = {2^3 * 4 - (3 % 2), 10 / 4 * 2}\n", [31, 5, 1]),
    ("solverName = 'EulerRoe'\nt = {}\nt.a = {b = 3}\nt.a.b = 16\nsize = {t.a.b, t['a'].b}\n", [16, 16, 1]),
    ("solverName = 'EulerRoe';;size = {8, [3] = 2, 4}\n", [8, 4, 2]),
])
def test_arithmetic_and_tables(hg, text, expect):
    st, cfg, msg = read(hg, text)
    assert st == 0, msg
    if expect is not None:
        assert list(cfg.size) == expect


REFUSED = [
    ("require 'util'\nsolverName = 'EulerRoe'\n", _abi.ERR_CONFIG, "line 1"),
    ("solverName = 'EulerRoe'\nif solverName == 'EulerRoe' then cfl = .1 end\n", _abi.ERR_CONFIG, "line 2"),
    ("solverName = 'EulerRoe'\nfunction calcSolid(x) return 0 end\n", _abi.ERR_CONFIG, "line 2"),
    ("solverName = 'EulerRoe'\ninitConds[initCondName].setup()\n", _abi.ERR_CONFIG, "line 2"),
    ("solverName = 'EulerRoe'\nlocal n = 4\n", _abi.ERR_CONFIG, "line 2"),
    ("solverName = 'EulerRoe'\nname = 'a' .. 'b'\n", _abi.ERR_CONFIG, "concatenation"),
    ("solverName = 'EulerRoe'\nslopeLimiter = 'Minmod'\n", _abi.ERR_CONFIG, "slope limiter"),
    ("solverName = 'EulerRoe'\nintegratorName = 'RK4'\n", _abi.ERR_CONFIG, "integrator"),
    ("solverName = 'EulerRoe'\nintegratorName = 'BackwardEulerConjugateGradient'\n", _abi.ERR_UNSUPPORTED, ""),
    ("solverName = 'EulerBurgers'\n", _abi.ERR_UNSUPPORTED, "EulerBurgers"),
    ("solverName = 'SRHDRoe'\n", _abi.ERR_CONFIG, "SRHDRoe"),
    ("size = {64, 64}\n", _abi.ERR_UNSUPPORTED, "solverName"),
    ("solverName = 'EulerRoe'\nboundaryMethods = {{min='OPEN', max='PERIODIC'}}\n", _abi.ERR_CONFIG, "OPEN"),
    ("solverName = 'EulerRoe'\nsize = {256.5, 256}\n", _abi.ERR_CONFIG, "integer"),
    ("solverName = 'EulerRoe'\nsize = 256\n", _abi.ERR_CONFIG, "table"),
    ("solverName = 'EulerRoe'\ncfl = 'fast'\n", _abi.ERR_CONFIG, "number"),
    ("solverName = 'EulerRoe'\ndefs.idealGas_heatCapacityRatio = 1.4\n", _abi.ERR_CONFIG, "not a table"),
    ("solverName = 'EulerRoe'\nx = y + 1\n", _abi.ERR_CONFIG, "arithmetic"),
    ("solverName = 'EulerRoe'\nname = 'open\n", _abi.ERR_CONFIG, "unfinished string"),
    ("solverName = 'EulerRoe'\n--[[ never closed\n", _abi.ERR_CONFIG, "long comment"),
    ("solverName = 'EulerRoe'\nsize = {64, 64\n", _abi.ERR_CONFIG, "'}' expected"),
    ("solverName = 'EulerRoe'\ngaussSeidelMaxIter = 1e12\n", _abi.ERR_CONFIG, "integer"),
    ("solverName = 'EulerRoe'\nx = 12abc\n", _abi.ERR_CONFIG, "malformed number"),
]


@pytest.mark.parametrize("text,status,needle", REFUSED)
def test_refused(hg, text, status, needle):
    before = _abi.make_config(solver="EulerHLL", size=(12, 10))
    cfg = _abi.make_config(solver="EulerHLL", size=(12, 10))
    st = hg.lib().hgpu_config_from_string(text.encode(), ctypes.byref(cfg))
    msg = hg.lib().hgpu_last_error().decode()
    assert st == status, (st, msg)
    assert needle in msg, msg
    assert fields(cfg) == fields(before)          # written only on success


def test_missing_file_and_null_arguments(hg, tmp_path):
    cfg = _abi.HgpuConfig()
    assert hg.lib().hgpu_config_from_file(str(tmp_path / "absent.lua").encode(), ctypes.byref(cfg)) == _abi.ERR_ARG
    assert hg.lib().hgpu_config_from_string(None, ctypes.byref(cfg)) == _abi.ERR_ARG
    assert hg.lib().hgpu_config_from_string(b"solverName = 'EulerRoe'", None) == _abi.ERR_ARG
