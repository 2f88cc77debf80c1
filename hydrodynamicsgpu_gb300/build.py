"""In-tree build of libhgpu.so (sm_103a) with nvcc, translation units compiled in parallel.

Kernel translation units are compiled with --fmad=false: the reference kernels'
a*b+c is two roundings, and the parity contract is bit-identical FP64 results.
Deliberately fused operations in the kernels call fma() explicitly.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhgpu.so")
# the checked variant (HGPU_CHECKED: index tests in the kernels, guard bands around
# every device allocation), built on request for the checked test suite
BUILD_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(PKG, "libhgpu_checked.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-I", os.path.join(REPO, "include"), "-I", CSRC]

SOURCES = {
    "kernels/roe.cu": ["--fmad=false"],
    "kernels/hllc.cu": ["--fmad=false"],
    "kernels/combine.cu": ["--fmad=false"],
    "kernels/probe.cu": ["--fmad=false"],
    "kernels/noalloc.cu": ["--fmad=false"],
    "kernels/batch.cu": ["--fmad=false"],
    "kernels/batch_flux.cu": ["--fmad=false"],
    "kernels/adjoint.cu": [],
    "kernels/roe_record.cu": ["--fmad=false"],
    "kernels/display.cu": ["--fmad=false"],
    "kernels/gravity.cu": ["--fmad=false"],
    "kernels/health.cu": ["--fmad=false"],
    "kernels/roe_fused.cu": ["--fmad=false"],
    "host/fits.cu": [],
    "host/adjoint.cu": [],
    "host/batch_solver.cu": [],
    "host/solver.cu": [],
    "host/capi.cu": [],
    "host/config_file.cu": [],
}
HEADERS = ["kernels/fp64ops.cuh", "kernels/common.cuh", "kernels/roe_cells.cuh", "kernels/hllc_cells.cuh",
           "kernels/combine_cells.cuh", "kernels/batch.h", "kernels/batch_common.cuh", "host/batch_solver.h", "kernels/roe.cuh", "kernels/reduce.cuh", "kernels/kernels.h", "host/solver.h",
           "kernels/adjoint.h", "host/adjoint.h",
           "kernels/limiter_dual.cuh", "host/fits.h", "kernels/gravity.h", "kernels/health.cuh",
           "kernels/tma.cuh"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra, verbose, build_dir=BUILD):
    obj = os.path.join(build_dir, src.replace("/", "_").replace(".cu", ".o"))
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
           [os.path.join(REPO, "include", "hgpu", "hgpu.h"), os.path.abspath(__file__)]
    if not _stale(obj, deps):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    if verbose and r.stderr.strip():
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, jobs=None, checked=False):
    build_dir, lib = (BUILD_CHECKED, LIB_CHECKED) if checked else (BUILD, LIB)
    flags = ["-DHGPU_CHECKED"] if checked else []
    os.makedirs(build_dir, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1] + flags, verbose, build_dir), SOURCES.items()))
    if _stale(lib, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
        os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, checked="--checked" in sys.argv))
