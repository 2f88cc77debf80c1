"""hydrodynamicsgpu_gb300 -- GB300-native finite-volume Euler update (HydroGPU's solver path).

The compute path is libhgpu.so: hand-written sm_103a CUDA kernels behind the C ABI
of include/hgpu/hgpu.h.  This module is a thin ctypes mirror of that ABI plus a
``Solver`` class with the reference's host interface (src/Solver/Solver.h:75-145):
``init()``, ``resetState()``, ``update()``, ``save()``.  There is no CPU fallback:
if libhgpu.so is missing or no GPU is present, the calls fail loudly.
"""
import ctypes
import os

import numpy as np

from . import _abi
from ._abi import (COMPAT_REF, COMPAT_SEAM, FP32, FP64, HgpuConfig, INTEGRATORS, LIMITERS,  # noqa: F401
                   SOLVERS, make_config)

PKG = os.path.dirname(os.path.abspath(__file__))
# HGPU_LIBRARY selects another build of the library (the checked one: libhgpu_checked.so)
LIB_PATH = os.environ.get("HGPU_LIBRARY") or os.path.join(PKG, "libhgpu.so")

# every entry point of include/hgpu/hgpu.h: name -> (restype, argtypes)
_P = ctypes.c_void_p
_CFG = ctypes.POINTER(HgpuConfig)
SIGNATURES = {
    "hgpu_config_default": (ctypes.c_int, [_CFG]),
    "hgpu_config_from_file": (ctypes.c_int, [ctypes.c_char_p, _CFG]),
    "hgpu_config_from_string": (ctypes.c_int, [ctypes.c_char_p, _CFG]),
    "hgpu_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "hgpu_last_error": (ctypes.c_char_p, []),
    "hgpu_create": (ctypes.c_int, [_CFG, ctypes.POINTER(_P)]),
    "hgpu_destroy": (ctypes.c_int, [_P]),
    "hgpu_get_shape": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_size_t)]),
    "hgpu_set_state": (ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    "hgpu_set_state_potential": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P, ctypes.c_size_t]),
    "hgpu_get_potential": (ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    "hgpu_get_state": (ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    "hgpu_update": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "hgpu_step": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "hgpu_update_host": (ctypes.c_int, [_P, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.POINTER(ctypes.c_double)]),
    "hgpu_last_dt": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double)]),
    "hgpu_synchronize": (ctypes.c_int, [_P]),
    "hgpu_health": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint32)]),
    "hgpu_set_health_mode": (ctypes.c_int, [_P, ctypes.c_int]),
    "hgpu_set_fused_stages": (ctypes.c_int, [_P, ctypes.c_int]),
    "hgpu_state_device_ptr": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "hgpu_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "hgpu_set_graphs": (ctypes.c_int, [_P, ctypes.c_int]),
    "hgpu_kernels_per_step": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    "hgpu_select_device": (ctypes.c_int, [ctypes.c_int]),
    "hgpu_timed_update": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "hgpu_profile_update": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "hgpu_fp64_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "hgpu_checked_status": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint32)]),
    "hgpu_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(_P)]),
    "hgpu_host_free": (ctypes.c_int, [_P]),
    "hgpu_cfl_timestep_noalloc": (ctypes.c_int, [_CFG, _P, ctypes.POINTER(ctypes.c_double), _P]),
    "hgpu_update_frozen_dt": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "hgpu_adjoint_step": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_double]),
    "hgpu_checkpoint_create": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "hgpu_checkpoint_create_taped": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_P)]),
    "hgpu_checkpoint_forward": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double)]),
    "hgpu_checkpoint_dts": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "hgpu_checkpoint_backward": (ctypes.c_int, [_P, _P, _P]),
    "hgpu_checkpoint_times": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "hgpu_checkpoint_destroy": (ctypes.c_int, [_P]),
    "hgpu_limiter_selftest": (ctypes.c_int, [ctypes.c_ulonglong, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]),
    "hgpu_fp64_selftest": (ctypes.c_int, [ctypes.c_ulonglong, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong),
                                          ctypes.POINTER(ctypes.c_longlong)]),
    "hgpu_display": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_size_t]),
    "hgpu_display_device": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "hgpu_save_fits": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]),
    "hgpu_batch_create": (ctypes.c_int, [_CFG, ctypes.c_int, ctypes.POINTER(_P)]),
    "hgpu_batch_destroy": (ctypes.c_int, [_P]),
    "hgpu_batch_info": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong),
                                       ctypes.POINTER(ctypes.c_int)]),
    "hgpu_batch_set_state": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t]),
    "hgpu_batch_get_state": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t]),
    "hgpu_batch_update": (ctypes.c_int, [_P, ctypes.c_int]),
    "hgpu_batch_step": (ctypes.c_int, [_P, ctypes.c_int]),
    "hgpu_batch_timed_update": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "hgpu_batch_dts": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "hgpu_batch_health": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint32)]),
    "hgpu_batch_problem_health": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint32), ctypes.c_int]),
    "hgpu_batch_get_tuning": (ctypes.c_int, [_P, _P]),
    "hgpu_batch_set_tuning": (ctypes.c_int, [_P, _P]),
    "hgpu_batch_autotune": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int]),
}


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_int), ("total_ms", ctypes.c_double)]


def config_from_file(path):
    """An HgpuConfig read from a config.lua-style settings file (hgpu_config_from_file)."""
    cfg = HgpuConfig()
    check(lib().hgpu_config_from_file(os.fsencode(path), ctypes.byref(cfg)))
    return cfg


def config_from_string(text):
    """An HgpuConfig read from the text of a config.lua-style settings file."""
    cfg = HgpuConfig()
    check(lib().hgpu_config_from_string(text.encode(), ctypes.byref(cfg)))
    return cfg


def select_device(device):
    check(lib().hgpu_select_device(int(device)))


def fp64_selftest(cases=1 << 26, seed=1):
    """(mul, div) mismatches of the integer-pipe binary64 product/quotient against the FP64 unit."""
    m, d = ctypes.c_longlong(), ctypes.c_longlong()
    check(lib().hgpu_fp64_selftest(int(seed), int(cases), ctypes.byref(m), ctypes.byref(d)))
    return m.value, d.value


def limiter_selftest(cases=1 << 26, seed=1):
    """Mismatches of the bit-pattern MinMod/Superbee against their fmin/fmax expressions."""
    m = ctypes.c_longlong()
    check(lib().hgpu_limiter_selftest(int(seed), int(cases), ctypes.byref(m)))
    return m.value


def fp64_peak():
    """Measured FP64 fma instructions per second of the current device."""
    r = ctypes.c_double()
    check(lib().hgpu_fp64_peak(ctypes.byref(r)))
    return r.value

class PinnedArray:
    """A numpy view of a page-locked host buffer (hgpu_host_alloc)."""

    def __init__(self, n, dtype):
        dtype = np.dtype(dtype)
        p = ctypes.c_void_p()
        check(lib().hgpu_host_alloc(n * dtype.itemsize, ctypes.byref(p)))
        self.ptr = p
        buf = (ctypes.c_char * (n * dtype.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=n)

    def free(self):
        if self.ptr:
            self.array = None
            lib().hgpu_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


_lib = None


class HgpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_abi.STATUS_NAMES.get(status, status), msg))
        self.status = status


def lib():
    """Load libhgpu.so (built in-tree by build()); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libhgpu.so not built: run __graft_entry__.build() or hydrodynamicsgpu_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != 0:
        raise HgpuError(status, lib().hgpu_last_error().decode())


class Solver:
    """A GB300 Euler solver (EulerRoe, EulerHLLC or EulerHLL) behind the C ABI.

    Mirrors the reference's host interface: construct with a config (the
    HydroGPUApp config fields), ``resetState(state)`` uploads an initial state
    (AoS, ghosts included), ``update(n)`` runs Solver::update n times, ``getState()``
    downloads it and ``save(directory)`` writes one FITS image per state channel."""

    def __init__(self, cfg=None, **kw):
        self.cfg = cfg if cfg is not None else make_config(**kw)
        h = ctypes.c_void_p()
        check(lib().hgpu_create(ctypes.byref(self.cfg), ctypes.byref(h)))
        self.h = h
        d, n, v = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        check(lib().hgpu_get_shape(self.h, ctypes.byref(d), ctypes.byref(n), ctypes.byref(v)))
        self.dim, self.num_states, self.volume = d.value, n.value, v.value
        self.dtype = np.float32 if self.cfg.precision == FP32 else np.float64
        self.frame = 0

    def close(self):
        if getattr(self, "h", None):
            lib().hgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def count(self):
        return self.volume * self.num_states

    def shape(self):
        s = self.cfg.size
        return (s[2], s[1], s[0], self.num_states)

    def name(self):
        return "EulerRoe" if self.cfg.solver == 0 else "EulerHLLC"

    def resetState(self, state, potential=None):
        """Solver::resetState's upload (Converter::toGPU + SelfGravitation::resetState):
        ``potential`` is the initial conditions' potential channel (one value per cell),
        or None for zero.  With use_gravity the potential starts as -density instead."""
        a = np.ascontiguousarray(state, dtype=self.dtype).reshape(-1)
        if a.size != self.count:
            raise ValueError("state has %d elements, solver needs %d" % (a.size, self.count))
        if potential is None:
            check(lib().hgpu_set_state(self.h, a.ctypes.data, a.size))
            return
        p = np.ascontiguousarray(potential, dtype=self.dtype).reshape(-1)
        if p.size != self.volume:
            raise ValueError("potential has %d elements, solver needs %d" % (p.size, self.volume))
        check(lib().hgpu_set_state_potential(self.h, a.ctypes.data, a.size, p.ctypes.data, p.size))

    def getPotential(self, out=None):
        """The gravitational potential (one value per cell, ghosts included)."""
        a = out if out is not None else np.empty(self.volume, dtype=self.dtype)
        check(lib().hgpu_get_potential(self.h, a.ctypes.data, a.size))
        return a

    get_potential = getPotential

    set_state = resetState

    def getState(self, out=None):
        a = out if out is not None else np.empty(self.count, dtype=self.dtype)
        check(lib().hgpu_get_state(self.h, a.ctypes.data, a.size))
        return a

    get_state = getState

    def update(self, nsteps=1, want_dt=True):
        dt = ctypes.c_double()
        check(lib().hgpu_update(self.h, int(nsteps), ctypes.byref(dt) if want_dt else None))
        self.frame += nsteps
        return dt.value if want_dt else None

    def update_host(self, state, nsteps=1, out=None):
        """hgpu_update_host: upload `state` (resetState), run `nsteps` updates and
        download the result into `out` (a new array if None; it may be `state`), the
        copies overlapped with the first and last step.  Returns (out, last dt).  Use
        PinnedArray buffers for the overlap."""
        a = state if (isinstance(state, np.ndarray) and state.dtype == self.dtype and state.flags.c_contiguous) \
            else np.ascontiguousarray(state, dtype=self.dtype)
        a = a.reshape(-1)
        o = out if out is not None else np.empty(self.count, dtype=self.dtype)
        if o.dtype != self.dtype or not o.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous %s array" % np.dtype(self.dtype).name)
        if a.size != self.count or o.size != self.count:
            raise ValueError("state has %d / out %d elements, solver needs %d" % (a.size, o.size, self.count))
        dt = ctypes.c_double()
        check(lib().hgpu_update_host(self.h, a.ctypes.data, a.size, int(nsteps), o.ctypes.data, o.size,
                                     ctypes.byref(dt)))
        self.frame += nsteps
        return o, dt.value

    def last_dt(self):
        dt = ctypes.c_double()
        check(lib().hgpu_last_dt(self.h, ctypes.byref(dt)))
        return dt.value

    def synchronize(self):
        check(lib().hgpu_synchronize(self.h))

    def set_health_mode(self, mode):
        """_abi.HEALTH_OFF / HEALTH_RECORD (default) / HEALTH_STRICT (hgpu_set_health_mode)."""
        check(lib().hgpu_set_health_mode(self.h, int(mode)))

    def health(self):
        f = ctypes.c_uint32()
        check(lib().hgpu_health(self.h, ctypes.byref(f)))
        return f.value

    def set_fused_stages(self, on):
        """Each Runge-Kutta stage as two fused per-direction kernels (2D FP64 EulerRoe)."""
        check(lib().hgpu_set_fused_stages(self.h, 1 if on else 0))

    def set_graphs(self, on):
        check(lib().hgpu_set_graphs(self.h, 1 if on else 0))

    def kernels_per_step(self):
        n = ctypes.c_int()
        check(lib().hgpu_kernels_per_step(self.h, ctypes.byref(n)))
        return n.value

    def timed_update(self, nsteps):
        """Run nsteps and return their device time in ms (CUDA events on the solver stream)."""
        ms = ctypes.c_float()
        check(lib().hgpu_timed_update(self.h, int(nsteps), ctypes.byref(ms)))
        self.frame += nsteps
        return ms.value

    def profile(self, nsteps=1):
        """Per-kernel device times of nsteps plain-launch updates: {name: (launches, total_ms)}."""
        arr = (KernelTime * 32)()
        n = ctypes.c_int()
        check(lib().hgpu_profile_update(self.h, int(nsteps), ctypes.cast(arr, ctypes.c_void_p), 32, ctypes.byref(n)))
        self.frame += nsteps
        return {arr[i].name.decode(): (arr[i].launches, arr[i].total_ms) for i in range(min(n.value, 32))}

    def state_device_ptr(self):
        p = ctypes.c_void_p()
        check(lib().hgpu_state_device_ptr(self.h, ctypes.byref(p)))
        return p.value

    def stream(self):
        p = ctypes.c_void_p()
        check(lib().hgpu_stream(self.h, ctypes.byref(p)))
        return p.value

    def update_frozen_dt(self, dts):
        """Advance len(dts) steps with the given dt per step (eigenbasis and stages as
        in update(), the CFL reduction replaced by the given value)."""
        a = np.ascontiguousarray(dts, dtype=np.float64)
        check(lib().hgpu_update_frozen_dt(self.h, a.size, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        self.frame += a.size

    def adjoint_step(self, d_u, d_lam_next, d_lam_out, dt):
        """lam_out = (d u^{n+1}/d u^n)^T lam_next for the step from u^n with dt; device
        pointers (ints) to full FP64 state arrays."""
        check(lib().hgpu_adjoint_step(self.h, ctypes.c_void_p(d_u), ctypes.c_void_p(d_lam_next),
                                      ctypes.c_void_p(d_lam_out), float(dt)))

    def save(self, directory="."):
        """Solver::save (src/Solver/Solver.cpp:549-589): <CHANNEL><index>.fits per state
        channel plus `potential`, 32-bit float images; returns the save index."""
        idx = ctypes.c_int()
        check(lib().hgpu_save_fits(self.h, str(directory).encode(), ctypes.byref(idx)))
        return idx.value

    def display(self, method):
        """convertToTex (res/EulerMHDCommon.cl:4-116): the display scalar of every cell
        as float32, shaped like the grid; `method` is a name of DISPLAY_NAMES(dim) or
        the reference's DISPLAY_* index."""
        m = _abi.display_index(self.dim, method)
        out = np.empty(self.count // self.num_states, dtype=np.float32)
        check(lib().hgpu_display(self.h, m, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), out.size))
        return out.reshape(self.shape()[:-1])


class BatchTuning(ctypes.Structure):
    _fields_ = [("tile_x", ctypes.c_int), ("tile_y", ctypes.c_int), ("tile_z", ctypes.c_int),
                ("staged", ctypes.c_int), ("blocks_per_sm", ctypes.c_int), ("split_flux", ctypes.c_int),
                ("cells_per_thread", ctypes.c_int)]


class Batch:
    """Many independent problems (same solver/dim/integrator/limiter/precision, their
    own sizes, domains, cfl and boundaries) advanced together in persistent launches."""

    def __init__(self, cfgs):
        arr = (HgpuConfig * len(cfgs))(*cfgs)
        self.cfgs = list(cfgs)
        h = ctypes.c_void_p()
        check(lib().hgpu_batch_create(arr, len(cfgs), ctypes.byref(h)))
        self.h = h
        self.dtype = np.float32 if cfgs[0].precision == FP32 else np.float64
        self.n = len(cfgs)

    def close(self):
        if getattr(self, "h", None):
            lib().hgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def count(self, p):
        return _abi.config_count(self.cfgs[p])

    def set_state(self, p, state):
        a = np.ascontiguousarray(state, dtype=self.dtype).reshape(-1)
        check(lib().hgpu_batch_set_state(self.h, int(p), a.ctypes.data, a.size))

    def get_state(self, p):
        a = np.empty(self.count(p), dtype=self.dtype)
        check(lib().hgpu_batch_get_state(self.h, int(p), a.ctypes.data, a.size))
        return a

    def update(self, nsteps=1):
        check(lib().hgpu_batch_update(self.h, int(nsteps)))

    def timed_update(self, nsteps):
        ms = ctypes.c_float()
        check(lib().hgpu_batch_timed_update(self.h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def dts(self):
        out = (ctypes.c_double * self.n)()
        check(lib().hgpu_batch_dts(self.h, out, self.n))
        return np.array(out[:])

    def health(self):
        f = ctypes.c_uint32()
        check(lib().hgpu_batch_health(self.h, ctypes.byref(f)))
        return f.value

    def problem_health(self):
        """Every problem's health bits since the last read (hgpu_batch_problem_health)."""
        n = len(self.cfgs)
        out = (ctypes.c_uint32 * n)()
        check(lib().hgpu_batch_problem_health(self.h, out, n))
        return np.array(out[:], dtype=np.uint32)

    def info(self):
        n, cells, k = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int()
        check(lib().hgpu_batch_info(self.h, ctypes.byref(n), ctypes.byref(cells), ctypes.byref(k)))
        return n.value, cells.value, k.value

    def tuning(self):
        t = BatchTuning()
        check(lib().hgpu_batch_get_tuning(self.h, ctypes.byref(t)))
        return (t.tile_x, t.tile_y, t.tile_z, t.staged, t.blocks_per_sm, t.split_flux, t.cells_per_thread)

    def set_tuning(self, tile=(32, 8, 1), staged=1, blocks_per_sm=0, split_flux=None, cells_per_thread=1):
        """split_flux None keeps the current choice (the two-pass flux for FP64 EulerRoe)."""
        if split_flux is None:
            split_flux = self.tuning()[5]
        t = BatchTuning(tile[0], tile[1], tile[2], staged, blocks_per_sm, split_flux, cells_per_thread)
        check(lib().hgpu_batch_set_tuning(self.h, ctypes.byref(t)))

    def autotune(self, cache_path=None, steps=2):
        check(lib().hgpu_batch_autotune(self.h, cache_path.encode() if cache_path else None, int(steps)))
        return self.tuning()


class Checkpoints:
    """Checkpointed trajectory of `nsteps` steps from the solver's current state
    (hgpu_checkpoint_*): forward() keeps every `every`-th state and each step's dt,
    backward() maps the cotangent of the final state to that of the initial state."""

    def __init__(self, solver, nsteps, every=None, taped=False):
        """taped: record every step's tape during forward() (hgpu_checkpoint_create_taped;
        memory for nsteps tapes), so backward() runs the reverse steps only."""
        h = ctypes.c_void_p()
        if taped:
            check(lib().hgpu_checkpoint_create_taped(solver.h, int(nsteps), ctypes.byref(h)))
        else:
            check(lib().hgpu_checkpoint_create(solver.h, int(nsteps), int(every), ctypes.byref(h)))
        self.h, self.solver, self.nsteps = h, solver, int(nsteps)

    def close(self):
        if getattr(self, "h", None):
            lib().hgpu_checkpoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, dts=None):
        if dts is None:
            check(lib().hgpu_checkpoint_forward(self.h, None))
        else:
            a = np.ascontiguousarray(dts, dtype=np.float64)
            if a.size != self.nsteps:
                raise ValueError("need %d dt values" % self.nsteps)
            check(lib().hgpu_checkpoint_forward(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))

    def dts(self):
        out = (ctypes.c_double * self.nsteps)()
        check(lib().hgpu_checkpoint_dts(self.h, out, self.nsteps))
        return np.array(out[:])

    def backward(self, d_lam_T, d_lam_0):
        check(lib().hgpu_checkpoint_backward(self.h, ctypes.c_void_p(d_lam_T), ctypes.c_void_p(d_lam_0)))

    def times(self):
        f, b = ctypes.c_float(), ctypes.c_float()
        check(lib().hgpu_checkpoint_times(self.h, ctypes.byref(f), ctypes.byref(b)))
        return f.value, b.value
