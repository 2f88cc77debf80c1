#!/usr/bin/env python3
"""Build "refcl": the reference's own OpenCL kernels compiled as C++ for the CPU.

TEST INFRASTRUCTURE ONLY.  The output is the strongest parity pin available here
(no CPU OpenCL runtime exists on either machine): the kernel sources of
KennethYeah/HydrodynamicsGPU (res/*.cl) are read from the reference checkout,
mechanically rewritten so that they are valid C++ (nothing else changes), and
assembled in the order Solver::getProgramSources builds the OpenCL program
(src/Solver/Solver.cpp:260-315, FiniteVolumeSolver.cpp:28-39, Roe.cpp:63-80,
SelfGravitationBehavior.h:47-52, EulerRoe.cpp:24-29, HLL.cpp:25-29).

Everything is written under oracle/_ref/ (git-ignored, never committed):
  _ref/gen/            rewritten kernel sources + one program per variant
  _ref/librefcl_*.so   one library per (solver, dim, precision)
When the reference checkout is absent (e.g. on the GPU host) an existing
_ref/gen/ is compiled as is.

Rewrites applied to copies of the .cl files:
  __kernel/__global/__local -> removed, __const -> const
  (int4)(..)/(int2)(..)/(real4)(..) vector literals -> make_int4(..)/make_int2(..)/make_real4(..)
  v.xy = v.yx; / v.xz = v.zx;  -> refcl_swap_xy(v); / refcl_swap_xz(v);
  program-scope `constant T name = init;` -> a static plus an init function
The program preamble's compile-time SIZE/STEP/DX values and the `defs` numbers
become runtime globals so one build serves every grid; DIM, NUM_STATES,
EULER_DIM and the real type stay compile-time, as they select #if branches.
res/EulerMHDCommon.cl is display-only (convertToTex, images) and is not built;
the VELOCITY macro it pulls in (res/include/HydroGPU/Euler.h) is included directly.
"""
import argparse
import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(REPO, "oracle", "_ref")
GEN = os.path.join(OUT, "gen")

KERNEL_FILES = ["SlopeLimiter", "Common", "CalcFluxDeriv", "RoeEigenfieldLinear", "Roe",
                "EulerRoe", "EulerHLLC", "EulerHLL", "SelfGravitation"]
HEADER_FILES = ["Roe.h", "Euler.h"]
LIMITERS = ["DonorCell", "LaxWendroff", "BeamWarming", "Fromm", "CHARM", "HCUS", "HQUICK",
            "Koren", "MinMod", "Oshker", "Ospre", "Smart", "Sweby", "UMIST", "VanAlbada1",
            "VanAlbada2", "VanLeer", "MonotizedCentral", "Superbee", "BarthJespersen"]
VARIANTS = [(solver, dim, prec) for solver in ("roe", "hllc", "hll") for dim in (1, 2, 3) for prec in ("f64", "f32")]


def rewrite(text, const_inits):
    text = re.sub(r"\b__kernel\b", "", text)
    text = re.sub(r"\b__global\b", "", text)
    text = re.sub(r"\b__local\b", "", text)
    text = re.sub(r"\b__const\b", "const", text)
    text = re.sub(r"\((int4|int2|real4|float4)\)\s*\(", r"make_\1(", text)
    text = re.sub(r"(\w+)\.xy\s*=\s*\1\.yx\s*;", r"refcl_swap_xy(\1);", text)
    text = re.sub(r"(\w+)\.xz\s*=\s*\1\.zx\s*;", r"refcl_swap_xz(\1);", text)

    def const_decl(m):
        typ, name, init = m.group(1), m.group(2), m.group(3)
        const_inits.append(name)
        return "static %s %s; static void refcl_init_%s() { %s = %s; }" % (typ, name, name, name, init)

    text = re.sub(r"^constant\s+(\w+)\s+(\w+)\s*=\s*(.+?);", const_decl, text, flags=re.M)
    return text


SHIM_COMMON_H = """#pragma once
/* replaces res/include/HydroGPU/Shared/Common.h for the C++ build: `real` comes from
   refcl_shim.h; the cell index layout is the reference's INDEX/INDEXV */
#define INDEX(a,b,c) ((a) + SIZE_X * ((b) + SIZE_Y * (c)))
#define INDEXV(i) INDEX((i).x, (i).y, (i).z)
"""


def generate(ref):
    res = os.path.join(ref, "res")
    if os.path.isdir(GEN):
        shutil.rmtree(GEN)
    os.makedirs(os.path.join(GEN, "include", "HydroGPU", "Shared"))
    const_inits = []
    for name in KERNEL_FILES:
        with open(os.path.join(res, name + ".cl")) as f:
            src = f.read()
        with open(os.path.join(GEN, name + ".cl.inc"), "w") as f:
            f.write("/* rewritten copy of res/%s.cl (see oracle/refcl/build_refcl.py) */\n" % name)
            f.write(rewrite(src, const_inits))
    for name in HEADER_FILES:
        with open(os.path.join(res, "include", "HydroGPU", name)) as f:
            src = f.read()
        with open(os.path.join(GEN, "include", "HydroGPU", name), "w") as f:
            f.write(rewrite(src, []))
    # the scalar display kernel (convertToTex) alone: the rest of the file draws vector-field geometry
    with open(os.path.join(res, "EulerMHDCommon.cl")) as f:
        src = f.read()
    display = src[src.index("__kernel void convertToTex("):src.index("constant float2 offset[6]")]
    with open(os.path.join(GEN, "EulerDisplay.cl.inc"), "w") as f:
        f.write("/* convertToTex of res/EulerMHDCommon.cl, rewritten (see oracle/refcl/build_refcl.py) */\n")
        f.write(re.sub(r"\bglobal\b", "", rewrite(display, const_inits)))   # `global` without underscores here
    with open(os.path.join(GEN, "include", "HydroGPU", "Shared", "Common.h"), "w") as f:
        f.write(SHIM_COMMON_H)
    for solver, dim, prec in VARIANTS:
        with open(os.path.join(GEN, "prog_%s_%dd_%s.cpp" % (solver, dim, prec)), "w") as f:
            f.write(program_source(solver, dim, prec, const_inits))


def program_source(solver, dim, prec, const_inits):
    n = dim + 2
    lines = ["/* generated by oracle/refcl/build_refcl.py: %s, dim %d, %s */" % (solver, dim, prec),
             "#define REFCL_REAL %s" % ("double" if prec == "f64" else "float"),
             '#include "refcl_shim.h"',
             "/* host headers first: the kernels #define gamma, which would rename struct fields */",
             '#include <vector>', '#include <limits>', '#include <algorithm>', '#include <omp.h>',
             '#include "hgpu/hgpu.h"']
    if solver == "roe":
        lines += ["#define REFCL_ROE 1", "#define SOLID 1"]
    lines += [
        "static int g_SIZE_X, g_SIZE_Y, g_SIZE_Z, g_STEP_X, g_STEP_Y, g_STEP_Z, g_STEP_W;",
        "static real g_DX, g_DY, g_DZ;",
        "static double g_gamma, g_G;",
        "static int g_limiter;",
        "#define DIM %d" % dim,
        "#define SIZE_X g_SIZE_X", "#define SIZE_Y g_SIZE_Y", "#define SIZE_Z g_SIZE_Z",
        "#define STEP_X g_STEP_X", "#define STEP_Y g_STEP_Y", "#define STEP_Z g_STEP_Z", "#define STEP_W g_STEP_W",
        "#define DX g_DX", "#define DY g_DY", "#define DZ g_DZ",
        "#define NUM_STATES %d" % n, "#define NUM_FLUX_STATES %d" % n,
        "#define idealGas_heatCapacityRatio ((real)g_gamma)",
        "#define selfGrav_gravitationalConstant ((real)g_G)",
    ]
    states = ["DENSITY", "MOMENTUM_X"] + (["MOMENTUM_Y"] if dim > 1 else []) + (["MOMENTUM_Z"] if dim > 2 else []) + ["ENERGY_TOTAL"]
    lines.append("enum {\n" + "".join("\tSTATE_%s,\n" % s for s in states) + "\tNUM_STATE\n};")
    lines.append("#define EULER_DIM %d" % dim)
    lines.append('#include "HydroGPU/Euler.h"')
    for lim in LIMITERS:
        lines += ["namespace refcl_lim_%s {" % lim, "#define SLOPE_LIMITER_%s" % lim,
                  '#include "SlopeLimiter.cl.inc"', "#undef SLOPE_LIMITER_%s" % lim, "}"]
    lines.append("typedef real (*refcl_limiter_fn)(real);")
    lines.append("static const refcl_limiter_fn refcl_limiters[%d] = {%s};" % (
        len(LIMITERS), ", ".join("refcl_lim_%s::slopeLimiter" % l for l in LIMITERS)))
    lines.append("real slopeLimiter(real r) { return refcl_limiters[g_limiter](r); }")
    lines += ['#include "Common.cl.inc"', '#include "CalcFluxDeriv.cl.inc"']
    if solver == "roe":
        lines += ["#define EIGEN_TRANSFORM_STRUCT_SIZE %d" % (2 * n * n), "#define EIGEN_SPACE_DIM %d" % n,
                  '#include "RoeEigenfieldLinear.cl.inc"', '#include "Roe.cl.inc"',
                  '#include "SelfGravitation.cl.inc"', '#include "EulerRoe.cl.inc"']
    elif solver == "hllc":
        lines += ['#include "EulerHLLC.cl.inc"', '#include "SelfGravitation.cl.inc"']
    else:
        lines += ['#include "EulerHLL.cl.inc"', '#include "SelfGravitation.cl.inc"']
    display = ["DENSITY", "VELOCITY", "VELOCITY_X"] + (["VELOCITY_Y"] if dim > 1 else []) + \
        (["VELOCITY_Z"] if dim > 2 else []) + ["PRESSURE", "ENERGY_INTERNAL", "ENERGY_KINETIC", "ENERGY_TOTAL",
                                               "POTENTIAL"]
    lines.append("enum {\n" + "".join("\tDISPLAY_%s,\n" % d for d in display) + "\tNUM_DISPLAY\n};")
    lines += ["#define DISPLAY_NONE -1", "#ifndef gamma", "#define gamma idealGas_heatCapacityRatio", "#endif",
              '#include "EulerDisplay.cl.inc"']
    names = sorted(set(const_inits))
    lines.append("static void refcl_init_constants() { %s }" % " ".join("refcl_init_%s();" % c for c in names))
    lines.append('#include "refcl_driver.inc"')
    return "\n".join(lines) + "\n"


def lib_path(solver, dim, prec):
    return os.path.join(OUT, "librefcl_%s_%dd_%s.so" % (solver, dim, prec))


def compile_variant(v, cxx="g++"):
    solver, dim, prec = v
    src = os.path.join(GEN, "prog_%s_%dd_%s.cpp" % v)
    out = lib_path(*v)
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-w", "-I", GEN, "-I", os.path.join(GEN, "include"), "-I", HERE, "-I", os.path.join(REPO, "include"),
           "-o", out + ".tmp", src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("refcl build failed for %s:\n%s" % (v, r.stderr[-4000:]))
    os.replace(out + ".tmp", out)
    return out


def build(ref=None, variants=None, jobs=None, quiet=True):
    """ref: the reference checkout (--ref, or the HGPU_REFERENCE_DIR environment
    variable); without one, an existing _ref/gen/ is compiled as is."""
    ref = ref or os.environ.get("HGPU_REFERENCE_DIR")
    if ref and os.path.isdir(os.path.join(ref, "res")):
        generate(ref)
    elif not os.path.isdir(GEN):
        if not quiet:
            print("refcl: no reference checkout and no generated sources; skipped")
        return []
    variants = variants or VARIANTS
    jobs = jobs or min(len(variants), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        outs = list(ex.map(compile_variant, variants))
    if not quiet:
        print("refcl: built %d libraries into %s" % (len(outs), OUT))
    return outs


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="the reference checkout (default: $HGPU_REFERENCE_DIR)")
    ap.add_argument("--jobs", type=int, default=None)
    args = ap.parse_args()
    build(args.ref, jobs=args.jobs, quiet=False)
