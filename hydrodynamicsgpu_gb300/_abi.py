"""ctypes mirror of include/hgpu/hgpu.h (types, enums and name registries).

The name registries are the string keys the reference reads from its Lua config:
solver names (src/HydroGPUApp.cpp:90-118), integrator names
(src/Solver/Solver.cpp:178-204), slope limiter names (res/SlopeLimiter.cl:5-68,
read from the key ``slopeLimiter`` at src/Solver/Solver.cpp:285-287) and boundary
method names (src/Equation/Euler.cpp:30-34, "NONE" at src/HydroGPUApp.cpp:505-507).
"""
import ctypes

HGPU_OK = 0
STATUS_NAMES = {
    0: "HGPU_OK", 1: "HGPU_ERR_CONFIG", 2: "HGPU_ERR_CUDA", 3: "HGPU_ERR_NONFINITE",
    4: "HGPU_ERR_TIMEOUT", 5: "HGPU_ERR_OOB", 6: "HGPU_ERR_ARG", 7: "HGPU_ERR_UNSUPPORTED",
    8: "HGPU_ERR_NOMEM", 9: "HGPU_ERR_UNPHYSICAL",
}
(OK, ERR_CONFIG, ERR_CUDA, ERR_NONFINITE, ERR_TIMEOUT, ERR_OOB, ERR_ARG, ERR_UNSUPPORTED, ERR_NOMEM,
 ERR_UNPHYSICAL) = range(10)
# health word bits (hgpu_health) and modes (hgpu_set_health_mode)
HEALTH_NONFINITE_DT, HEALTH_HLLC_NOBRANCH, HEALTH_STATE_NONFINITE, HEALTH_STATE_DENSITY, HEALTH_STATE_PRESSURE = \
    1, 2, 4, 8, 16
HEALTH_COPY_TIMEOUT = 32
HEALTH_OFF, HEALTH_RECORD, HEALTH_STRICT = 0, 1, 2

SOLVERS = {"EulerRoe": 0, "EulerHLLC": 1, "EulerHLL": 2}
BOUNDARIES = {"NONE": -1, "PERIODIC": 0, "MIRROR": 1, "FREEFLOW": 2}
LIMITERS = ["DonorCell", "LaxWendroff", "BeamWarming", "Fromm", "CHARM", "HCUS", "HQUICK",
            "Koren", "MinMod", "Oshker", "Ospre", "Smart", "Sweby", "UMIST", "VanAlbada1",
            "VanAlbada2", "VanLeer", "MonotizedCentral", "Superbee", "BarthJespersen"]
INTEGRATORS = ["ForwardEuler", "RungeKutta2", "RungeKutta2Heun", "RungeKutta2Ralston", "RungeKutta3",
               "RungeKutta4", "RungeKutta4_3_8thsRule", "RungeKutta2TVD", "RungeKutta2NonTVD",
               "RungeKutta3TVD", "RungeKutta4TVD", "RungeKutta4NonTVD"]
INTEGRATOR_ORDER = [1, 2, 2, 2, 3, 4, 4, 2, 2, 3, 4, 4]
FP64, FP32 = 0, 1
COMPAT_REF, COMPAT_SEAM = 0, 1


class HgpuConfig(ctypes.Structure):
    _fields_ = [
        ("solver", ctypes.c_int),
        ("dim", ctypes.c_int),
        ("size", ctypes.c_int * 3),
        ("xmin", ctypes.c_double * 3),
        ("xmax", ctypes.c_double * 3),
        ("gamma", ctypes.c_double),
        ("cfl", ctypes.c_float),
        ("use_fixed_dt", ctypes.c_int),
        ("fixed_dt", ctypes.c_double),
        ("boundary", (ctypes.c_int * 2) * 3),
        ("limiter", ctypes.c_int),
        ("integrator", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("compat", ctypes.c_int),
        ("use_gravity", ctypes.c_int),
        ("gauss_seidel_max_iter", ctypes.c_int),
        ("gravitational_constant", ctypes.c_double),
        ("reserved", ctypes.c_int * 4),
    ]


def _index(name, table, what):
    if isinstance(name, int):
        return name
    if isinstance(table, dict):
        if name not in table:
            raise ValueError("unknown %s %r" % (what, name))
        return table[name]
    if name not in table:
        raise ValueError("unknown %s %r" % (what, name))
    return table.index(name)


def make_config(solver="EulerRoe", size=(256, 256), xmin=(-.5, -.5, -.5), xmax=(.5, .5, .5), gamma=1.4,
                cfl=.5, use_fixed_dt=False, fixed_dt=.001, boundary="FREEFLOW", limiter="Superbee",
                integrator="ForwardEuler", precision=FP64, compat=COMPAT_REF, dim=0, use_gravity=False,
                gauss_seidel_max_iter=20, gravitational_constant=1.):
    """Build an HgpuConfig from the reference's config key values.

    ``size`` lists cells per axis including the 2 ghost layers per side (the
    reference's ``size`` key); missing axes are 1.  ``boundary`` is one name for
    every side, or a sequence of per-axis ``{"min": name, "max": name}`` dicts /
    ``(min, max)`` pairs (the reference's ``boundaryMethods`` table).
    ``use_gravity``, ``gauss_seidel_max_iter`` and ``gravitational_constant`` are
    the ``useGravity``, ``gaussSeidelMaxIter`` and ``defs.selfGrav_gravitationalConstant``
    keys (res/config.lua:65-74)."""
    cfg = HgpuConfig()
    cfg.solver = _index(solver, SOLVERS, "solver")
    cfg.dim = dim
    size = list(size) + [1] * (3 - len(size))
    xmin = list(xmin) + [-.5] * (3 - len(xmin))
    xmax = list(xmax) + [.5] * (3 - len(xmax))
    for i in range(3):
        cfg.size[i] = int(size[i])
        cfg.xmin[i] = float(xmin[i])
        cfg.xmax[i] = float(xmax[i])
    cfg.gamma = float(gamma)
    cfg.cfl = float(cfl)
    cfg.use_fixed_dt = int(bool(use_fixed_dt))
    cfg.fixed_dt = float(fixed_dt)
    if isinstance(boundary, (str, int)):
        boundary = [(boundary, boundary)] * 3
    for i in range(3):
        b = boundary[i] if i < len(boundary) else ("NONE", "NONE")
        if isinstance(b, dict):
            b = (b.get("min", "NONE"), b.get("max", "NONE"))
        cfg.boundary[i][0] = _index(b[0], BOUNDARIES, "boundary method")
        cfg.boundary[i][1] = _index(b[1], BOUNDARIES, "boundary method")
    cfg.limiter = _index(limiter, LIMITERS, "slope limiter")
    cfg.integrator = _index(integrator, INTEGRATORS, "integrator")
    cfg.precision = int(precision)
    cfg.compat = int(compat)
    cfg.use_gravity = int(bool(use_gravity))
    cfg.gauss_seidel_max_iter = int(gauss_seidel_max_iter)
    cfg.gravitational_constant = float(gravitational_constant)
    return cfg


def config_dim(cfg):
    if cfg.dim:
        return cfg.dim
    for d in (3, 2, 1):
        if cfg.size[d - 1] > 1:
            return d
    return 0


def config_volume(cfg):
    return int(cfg.size[0]) * int(cfg.size[1]) * int(cfg.size[2])


def config_count(cfg):
    return config_volume(cfg) * (config_dim(cfg) + 2)


def display_names(dim):
    """The reference's DISPLAY_* enum for Euler in `dim` dimensions (Euler.cpp:18-27)."""
    return (["DENSITY", "VELOCITY", "VELOCITY_X"] + (["VELOCITY_Y"] if dim > 1 else []) +
            (["VELOCITY_Z"] if dim > 2 else []) +
            ["PRESSURE", "ENERGY_INTERNAL", "ENERGY_KINETIC", "ENERGY_TOTAL", "POTENTIAL"])


def display_index(dim, method):
    if isinstance(method, str):
        names = display_names(dim)
        if method.upper() not in names:
            raise ValueError("unknown display method %r for dim %d" % (method, dim))
        return names.index(method.upper())
    return int(method)
