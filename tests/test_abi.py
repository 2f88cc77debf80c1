"""The C ABI library: loads without a GPU, exports every declared entry point, and
its host-only calls work; compute calls fail loudly when no GPU is present."""
import ctypes
import os
import re

import pytest

import hydrodynamicsgpu_gb300 as hgmod
from hydrodynamicsgpu_gb300 import _abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for root, _, files in os.walk(os.path.join(REPO, "include")):
        for f in files:
            if f.endswith(".h"):
                text = open(os.path.join(root, f)).read()
                names += re.findall(r"^\s*(?:int|const char\*|double|void)\s+\**(hgpu_\w+)\s*\(", text, re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    assert len(declared_functions()) >= 20


def test_library_exports_every_declared_symbol(hg):
    L = hg.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert sorted(declared_functions()) == sorted(hgmod.SIGNATURES)


def test_config_default_and_status_strings(hg):
    cfg = _abi.HgpuConfig()
    assert hg.lib().hgpu_config_default(cfg) == 0
    assert list(cfg.size) == [256, 256, 1]
    assert abs(cfg.cfl - .5) == 0 and cfg.limiter == _abi.LIMITERS.index("Superbee")
    assert cfg.integrator == 0 and cfg.fixed_dt == .001
    for code, name in _abi.STATUS_NAMES.items():
        assert hg.lib().hgpu_status_string(code).decode() == name


def test_struct_layout_matches_header():
    import ctypes
    # offsets as laid out by a C compiler for include/hgpu/hgpu.h (x86-64 and aarch64 agree)
    assert ctypes.sizeof(_abi.HgpuConfig) == 168
    assert _abi.HgpuConfig.boundary.offset == 96 and _abi.HgpuConfig.reserved.offset == 136


def test_null_arguments_rejected(hg):
    L = hg.lib()
    assert L.hgpu_create(None, None) == 6
    assert L.hgpu_update(None, 1, None) == 6
    assert L.hgpu_destroy(None) == 0


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure mode")
def test_no_silent_cpu_fallback(hg):
    with pytest.raises(hgmod.HgpuError):
        hgmod.Solver(size=(16, 16))


def test_batch_rejects_mixed_configs(hg):
    """Batch validation runs before any device work: mixed solvers, dims or
    integrators and the SEAM scheme are refused with a status code."""
    codes = {v: k for k, v in _abi.STATUS_NAMES.items()}
    a = _abi.make_config(solver="EulerRoe", size=(20, 20))
    for other in (_abi.make_config(solver="EulerHLLC", size=(20, 20)),
                  _abi.make_config(solver="EulerRoe", size=(20, 20), integrator="RungeKutta4"),
                  _abi.make_config(solver="EulerRoe", size=(20,))):
        arr = (_abi.HgpuConfig * 2)(a, other)
        h = ctypes.c_void_p()
        assert hg.lib().hgpu_batch_create(arr, 2, ctypes.byref(h)) == codes["HGPU_ERR_CONFIG"]
        assert not h.value
    seam = _abi.make_config(solver="EulerRoe", size=(20, 20), compat=_abi.COMPAT_SEAM)
    arr = (_abi.HgpuConfig * 1)(seam)
    h = ctypes.c_void_p()
    assert hg.lib().hgpu_batch_create(arr, 1, ctypes.byref(h)) == codes["HGPU_ERR_UNSUPPORTED"]
    assert hg.lib().hgpu_batch_create(arr, 0, ctypes.byref(h)) == codes["HGPU_ERR_ARG"]
