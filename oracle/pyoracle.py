"""Python binding of the CPU oracles.  TEST INFRASTRUCTURE ONLY.

Two checkers of the HydroGPU Euler step, both run on the host CPU:
  * ``Oracle``  -- oracle/hydro_oracle.c, a plain-C restatement of the reference
                   kernels and host order (liboracle.so).
  * ``Refcl``   -- the reference's own OpenCL kernels compiled as C++
                   (oracle/refcl/build_refcl.py -> oracle/_ref/librefcl_*.so),
                   available wherever oracle/_ref/ was built.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may use this.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
from hydrodynamicsgpu_gb300 import _abi  # noqa: E402

LIB_ORACLE = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


def build_oracle(force=False):
    src = [os.path.join(HERE, "hydro_oracle.c"), os.path.join(HERE, "oracle_impl.h"),
           os.path.join(REPO, "include", "hgpu", "hgpu.h")]
    if not force and os.path.exists(LIB_ORACLE) and all(os.path.getmtime(LIB_ORACLE) >= os.path.getmtime(s) for s in src):
        return LIB_ORACLE
    cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB_ORACLE + ".tmp", src[0], "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB_ORACLE + ".tmp", LIB_ORACLE)
    return LIB_ORACLE


def build_refcl(quiet=True, ref=None):
    sys.path.insert(0, os.path.join(HERE, "refcl"))
    import build_refcl  # noqa
    return build_refcl.build(ref=ref, quiet=quiet)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = ctypes.CDLL(LIB_ORACLE)
        P = ctypes.POINTER(_abi.HgpuConfig)
        L.oracle_resolve.argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.oracle_create.argtypes = [P, ctypes.POINTER(ctypes.c_void_p)]
        L.oracle_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_set_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        L.oracle_set_state_potential.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                 ctypes.c_void_p, ctypes.c_size_t]
        L.oracle_get_potential.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        L.oracle_get_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        L.oracle_update.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_int)]
        L.oracle_get_buffer.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t]
        L.oracle_get_buffer.restype = ctypes.c_size_t
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def resolve(cfg):
    """(dim, baked dx[3], baked gamma, baked G) exactly as the reference program preamble bakes them."""
    d = ctypes.c_int()
    dx = (ctypes.c_double * 3)()
    g = ctypes.c_double()
    G = ctypes.c_double()
    st = lib().oracle_resolve(ctypes.byref(cfg), ctypes.byref(d), dx, ctypes.byref(g), ctypes.byref(G))
    if st:
        raise ValueError("invalid config: %s" % _abi.STATUS_NAMES.get(st, st))
    return d.value, [dx[0], dx[1], dx[2]], g.value, G.value


def set_threads(n):
    lib().oracle_set_threads(int(n))


def max_threads():
    return lib().oracle_max_threads()


# Grids below this many cells run single-threaded: an OpenMP parallel region per kernel
# costs more than the work of a small grid (and far more on a loaded machine).
SMALL_GRID_CELLS = 1 << 16


class _OneThread:
    """Context: the library's OpenMP thread count is 1 inside, restored after."""

    def __init__(self, get, put, active):
        self.get, self.put, self.active = get, put, active

    def __enter__(self):
        if self.active:
            self.prev = self.get()
            self.put(1)

    def __exit__(self, *exc):
        if self.active:
            self.put(self.prev)


class _Base:
    dtype = np.float64

    def _small(self):
        return _abi.config_volume(self.cfg) < SMALL_GRID_CELLS

    def _np(self):
        return np.float32 if self.cfg.precision == _abi.FP32 else np.float64

    @property
    def count(self):
        return _abi.config_volume(self.cfg) * (self.dim + 2)

    def shape(self):
        s = self.cfg.size
        return (s[2], s[1], s[0], self.dim + 2)


class Oracle(_Base):
    """Plain-C restatement (hydro_oracle.c)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.dim, self.dx, self.gamma, self.G = resolve(cfg)
        h = ctypes.c_void_p()
        st = lib().oracle_create(ctypes.byref(cfg), ctypes.byref(h))
        if st:
            raise ValueError("oracle_create: %s" % _abi.STATUS_NAMES.get(st, st))
        self.h = h
        self.last_dt = None
        self.nonfinite = False

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def set_state(self, a, potential=None):
        a = np.ascontiguousarray(a, dtype=self._np()).reshape(-1)
        assert a.size == self.count
        with self._threads():
            if potential is None:
                st = lib().oracle_set_state(self.h, a.ctypes.data, a.size)
            else:
                p = np.ascontiguousarray(potential, dtype=self._np()).reshape(-1)
                st = lib().oracle_set_state_potential(self.h, a.ctypes.data, a.size, p.ctypes.data, p.size)
        assert st == 0

    def _threads(self):
        return _OneThread(lib().oracle_max_threads, lib().oracle_set_threads, self._small())

    def get_potential(self):
        a = np.empty(_abi.config_volume(self.cfg), dtype=self._np())
        assert lib().oracle_get_potential(self.h, a.ctypes.data, a.size) == 0
        return a

    def get_state(self):
        a = np.empty(self.count, dtype=self._np())
        st = lib().oracle_get_state(self.h, a.ctypes.data, a.size)
        assert st == 0
        return a

    def update(self, nsteps=1):
        dt = ctypes.c_double()
        bad = ctypes.c_int()
        with self._threads():
            lib().oracle_update(self.h, int(nsteps), ctypes.byref(dt), ctypes.byref(bad))
        self.last_dt = dt.value
        self.nonfinite = bool(bad.value)
        return dt.value

    def display(self, method):
        """convertToTex restated: the display scalar of every cell (DISPLAY_* index)."""
        lib().oracle_display.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        return _display(lib().oracle_display, self.h, _abi.config_volume(self.cfg), method)

    def get_buffer(self, name):
        n = lib().oracle_get_buffer(self.h, name.encode(), None, 0)
        a = np.empty(n, dtype=self._np())
        lib().oracle_get_buffer(self.h, name.encode(), a.ctypes.data, n)
        return a


def refcl_available(cfg=None):
    if cfg is None:
        return os.path.exists(os.path.join(REF_DIR, "librefcl_roe_2d_f64.so"))
    return os.path.exists(_refcl_path(cfg))


def _refcl_path(cfg):
    dim = _abi.config_dim(cfg)
    return os.path.join(REF_DIR, "librefcl_%s_%dd_%s.so" % (
        ("roe", "hllc", "hll")[cfg.solver], dim, "f32" if cfg.precision == _abi.FP32 else "f64"))


_refcl_libs = {}


def _refcl_lib(path):
    if path not in _refcl_libs:
        L = ctypes.CDLL(path)
        L.refcl_create.argtypes = [ctypes.POINTER(_abi.HgpuConfig), ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                   ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_void_p)]
        L.refcl_set_state_potential.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                ctypes.c_void_p, ctypes.c_size_t]
        L.refcl_get_potential.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        L.refcl_destroy.argtypes = [ctypes.c_void_p]
        L.refcl_set_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        L.refcl_get_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        L.refcl_update.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.refcl_get_buffer.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t]
        L.refcl_get_buffer.restype = ctypes.c_size_t
        L.refcl_set_threads.argtypes = [ctypes.c_int]
        L.refcl_max_threads.restype = ctypes.c_int
        _refcl_libs[path] = L
    return _refcl_libs[path]


def _display(fn, h, count, method):
    out = np.empty(count, dtype=np.float32)
    st = fn(h, int(method), out.ctypes.data)
    if st:
        raise ValueError("display method %r: status %d" % (method, st))
    return out


class Refcl(_Base):
    """The reference's kernels compiled for the CPU (one active handle per variant library)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.dim, self.dx, self.gamma, self.G = resolve(cfg)
        path = _refcl_path(cfg)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.L = _refcl_lib(path)
        dx = (ctypes.c_double * 3)(*self.dx)
        h = ctypes.c_void_p()
        st = self.L.refcl_create(ctypes.byref(cfg), self.dim, dx, self.gamma, self.G, ctypes.byref(h))
        if st:
            raise ValueError("refcl_create: %d" % st)
        self.h = h
        self.last_dt = None

    def __del__(self):
        if getattr(self, "h", None):
            self.L.refcl_destroy(self.h)
            self.h = None

    def _threads(self):
        return _OneThread(self.L.refcl_max_threads, self.L.refcl_set_threads, self._small())

    def set_state(self, a, potential=None):
        a = np.ascontiguousarray(a, dtype=self._np()).reshape(-1)
        with self._threads():
            if potential is None:
                assert self.L.refcl_set_state(self.h, a.ctypes.data, a.size) == 0
            else:
                p = np.ascontiguousarray(potential, dtype=self._np()).reshape(-1)
                assert self.L.refcl_set_state_potential(self.h, a.ctypes.data, a.size, p.ctypes.data, p.size) == 0

    def get_potential(self):
        a = np.empty(_abi.config_volume(self.cfg), dtype=self._np())
        assert self.L.refcl_get_potential(self.h, a.ctypes.data, a.size) == 0
        return a

    def get_state(self):
        a = np.empty(self.count, dtype=self._np())
        assert self.L.refcl_get_state(self.h, a.ctypes.data, a.size) == 0
        return a

    def update(self, nsteps=1):
        dt = ctypes.c_double()
        with self._threads():
            self.L.refcl_update(self.h, int(nsteps), ctypes.byref(dt))
        self.last_dt = dt.value
        return dt.value

    def display(self, method):
        """convertToTex of every cell (the reference's DISPLAY_* index)."""
        self.L.refcl_display.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        return _display(self.L.refcl_display, self.h, _abi.config_volume(self.cfg), method)

    def get_buffer(self, name):
        n = self.L.refcl_get_buffer(self.h, name.encode(), None, 0)
        a = np.empty(n, dtype=self._np())
        self.L.refcl_get_buffer(self.h, name.encode(), a.ctypes.data, n)
        return a

    def set_threads(self, n):
        self.L.refcl_set_threads(int(n))

    def max_threads(self):
        return self.L.refcl_max_threads()
