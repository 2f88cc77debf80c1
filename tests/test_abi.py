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


def test_struct_layout_matches_header(tmp_path):
    # offsets as laid out by a C compiler for include/hgpu/hgpu.h (x86-64 and aarch64 agree)
    assert ctypes.sizeof(_abi.HgpuConfig) == 168
    assert _abi.HgpuConfig.boundary.offset == 96 and _abi.HgpuConfig.use_gravity.offset == 136
    assert _abi.HgpuConfig.gravitational_constant.offset == 144 and _abi.HgpuConfig.reserved.offset == 152
    # and every field against the C compiler itself
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    names = [f[0] for f in _abi.HgpuConfig._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "hgpu/hgpu.h"\nint main(void) {\n'
                   + "".join('printf("%%zu\\n", offsetof(hgpu_config, %s));\n' % n for n in names)
                   + 'printf("%zu\\n", sizeof(hgpu_config));\nreturn 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    want = [getattr(_abi.HgpuConfig, n).offset for n in names] + [ctypes.sizeof(_abi.HgpuConfig)]
    assert got == want


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


def test_gravity_combinations_refused(hg):
    """Self-gravity runs on the single-problem REF path; the batch, the SEAM scheme and
    the allocation-free timestep refuse it before any device work."""
    codes = {v: k for k, v in _abi.STATUS_NAMES.items()}
    grav = _abi.make_config(solver="EulerRoe", size=(20, 20), use_gravity=True)
    arr = (_abi.HgpuConfig * 1)(grav)
    h = ctypes.c_void_p()
    assert hg.lib().hgpu_batch_create(arr, 1, ctypes.byref(h)) == codes["HGPU_ERR_UNSUPPORTED"]
    seam = _abi.make_config(solver="EulerRoe", size=(20, 20), use_gravity=True, compat=_abi.COMPAT_SEAM)
    assert hg.lib().hgpu_create(ctypes.byref(seam), ctypes.byref(h)) == codes["HGPU_ERR_UNSUPPORTED"]
    dt = ctypes.c_double()
    assert hg.lib().hgpu_cfl_timestep_noalloc(ctypes.byref(grav), ctypes.c_void_p(1), ctypes.byref(dt),
                                              None) == codes["HGPU_ERR_UNSUPPORTED"]
    bad = _abi.make_config(solver="EulerRoe", size=(20, 20), use_gravity=True, gauss_seidel_max_iter=-1)
    assert hg.lib().hgpu_create(ctypes.byref(bad), ctypes.byref(h)) == codes["HGPU_ERR_CONFIG"]


def test_config_default_gravity_keys(hg):
    cfg = _abi.HgpuConfig()
    assert hg.lib().hgpu_config_default(cfg) == 0
    assert cfg.use_gravity == 0 and cfg.gauss_seidel_max_iter == 20 and cfg.gravitational_constant == 1.
