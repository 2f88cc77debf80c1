#!/usr/bin/env python3
"""Generate the golden fixtures of tests/golden/ from the reference's own kernels.

The fixtures are produced by "refcl": HydroGPU's OpenCL kernels (res/*.cl),
compiled for the CPU by oracle/refcl/build_refcl.py and driven in the reference
host order.  Each fixture stores the configuration, the seeded initial state, the
dt of every step and the state after the last step.  Run from the repository
root in a checkout where oracle/_ref/ can be built (the reference sources are
needed once):

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

from hydrodynamicsgpu_gb300 import _abi  # noqa: E402
from hydrodynamicsgpu_gb300 import initconds as ic  # noqa: E402


def blocky(size, dim, seed):
    shape = tuple(reversed(list(size) + [1] * (3 - len(size))))
    rng = np.random.default_rng(seed)
    rho = np.round(rng.uniform(.5, 2., shape) * 2) / 2
    p = np.round(rng.uniform(.5, 2., shape) * 2) / 2
    v = [np.round(rng.uniform(-.5, .5, shape) * 4) / 4 for _ in range(3)]
    return ic.build_state_euler(dim, 1.4, rho, v[0], v[1], v[2], p)


CASES = [
    dict(name="sod_roe_fe_superbee_freeflow_1d", steps=20,
         cfg=dict(solver="EulerRoe", size=(64,), xmin=(0.,), xmax=(1.,), boundary="FREEFLOW", limiter="Superbee",
                  integrator="ForwardEuler", cfl=.5),
         init=lambda: ic.sod(size=(64,))),
    dict(name="kh_roe_rk4_minmod_periodic_2d", steps=5,
         cfg=dict(solver="EulerRoe", size=(32, 32), boundary="PERIODIC", limiter="MinMod", integrator="RungeKutta4",
                  cfl=.5),
         init=lambda: ic.kelvin_helmholtz(size=(32, 32), seed=0)),
    dict(name="quad5_roe_rk2_superbee_freeflow_2d", steps=5,
         cfg=dict(solver="EulerRoe", size=(24, 24), boundary="FREEFLOW", limiter="Superbee",
                  integrator="RungeKutta2", cfl=.475),
         init=lambda: ic.configuration(5, size=(24, 24))),
    dict(name="kh_hllc_rk4_periodic_2d", steps=5,
         cfg=dict(solver="EulerHLLC", size=(32, 32), boundary="PERIODIC", limiter="MinMod", integrator="RungeKutta4",
                  cfl=.5),
         init=lambda: ic.kelvin_helmholtz(size=(32, 32), seed=1)),
    dict(name="grf_hllc_tvdrk2_mirror_3d", steps=3,
         cfg=dict(solver="EulerHLLC", size=(12, 12, 12), xmin=(0, 0, 0), xmax=(1, 1, 1), gamma=5. / 3.,
                  boundary="MIRROR", limiter="VanLeer", integrator="RungeKutta2TVD", cfl=.4),
         init=lambda: ic.lognormal_grf(size=(12, 12, 12), corr_cells=3.0, seed=1)),
    dict(name="quad3_hll_rk2heun_freeflow_2d", steps=5,
         cfg=dict(solver="EulerHLL", size=(24, 24), boundary="FREEFLOW", limiter="MinMod",
                  integrator="RungeKutta2Heun", cfl=.5),
         init=lambda: ic.configuration(3, size=(24, 24))),
    dict(name="sod_hll_rk4_mirror_1d", steps=10,
         cfg=dict(solver="EulerHLL", size=(64,), xmin=(0.,), xmax=(1.,), boundary="MIRROR", limiter="MinMod",
                  integrator="RungeKutta4", cfl=.5),
         init=lambda: ic.sod(size=(64,))),
    dict(name="roe_rk3tvd_umist_mirror_3d", steps=3,
         cfg=dict(solver="EulerRoe", size=(10, 9, 8), boundary="MIRROR", limiter="UMIST",
                  integrator="RungeKutta3TVD", cfl=.4),
         init=lambda: ic.lognormal_grf(size=(10, 9, 8), corr_cells=2.0, seed=4, gamma=1.4)),
    dict(name="roe_rk4tvd_koren_mirror_2d", steps=3,
         cfg=dict(solver="EulerRoe", size=(20, 18), boundary="MIRROR", limiter="Koren", integrator="RungeKutta4TVD"),
         init=lambda: ic.configuration(3, size=(20, 18))),
    dict(name="roe_fe_vanleer_degenerate_2d", steps=1,
         cfg=dict(solver="EulerRoe", size=(16, 14), boundary="FREEFLOW", limiter="VanLeer",
                  integrator="ForwardEuler"),
         init=lambda: blocky((16, 14), 2, 3)),
    dict(name="kh_roe_rk4_minmod_periodic_2d_fp32", steps=5,
         cfg=dict(solver="EulerRoe", size=(32, 32), boundary="PERIODIC", limiter="MinMod", integrator="RungeKutta4",
                  cfl=.5, precision=_abi.FP32),
         init=lambda: ic.kelvin_helmholtz(size=(32, 32), seed=0, dtype=np.float32)),
    # self-gravity (useGravity): Poisson relaxation at reset and in every callback
    dict(name="blobs_roe_rk2_gravity_periodic_2d", steps=3,
         cfg=dict(solver="EulerRoe", size=(24, 24), boundary="PERIODIC", limiter="MinMod", integrator="RungeKutta2",
                  use_gravity=True, gauss_seidel_max_iter=5, gravitational_constant=1.),
         init=lambda: ic.gravity_blobs(size=(24, 24), seed=7)),
    dict(name="blobs_roe_rk2_gravity_periodic_2d_fp32", steps=3,
         cfg=dict(solver="EulerRoe", size=(24, 24), boundary="PERIODIC", limiter="MinMod", integrator="RungeKutta2",
                  use_gravity=True, gauss_seidel_max_iter=5, gravitational_constant=1., precision=_abi.FP32),
         init=lambda: ic.gravity_blobs(size=(24, 24), seed=7, dtype=np.float32)),
    dict(name="blobs_hllc_fe_gravity_freeflow_1d", steps=5,
         cfg=dict(solver="EulerHLLC", size=(48,), boundary="FREEFLOW", integrator="ForwardEuler",
                  use_gravity=True, gauss_seidel_max_iter=10, gravitational_constant=.5),
         init=lambda: ic.gravity_blobs(size=(48,), seed=8)),
    dict(name="blobs_hll_rk4_gravity_mirror_3d", steps=2,
         cfg=dict(solver="EulerHLL", size=(10, 10, 10), boundary="MIRROR", integrator="RungeKutta4",
                  use_gravity=True, gauss_seidel_max_iter=2, gravitational_constant=1.),
         init=lambda: ic.gravity_blobs(size=(10, 10, 10), seed=9)),
    # a static potential channel without useGravity (the initial conditions' potential)
    dict(name="static_potential_roe_rk3tvd_freeflow_2d", steps=3,
         cfg=dict(solver="EulerRoe", size=(20, 20), boundary="FREEFLOW", limiter="Superbee",
                  integrator="RungeKutta3TVD"),
         init=lambda: ic.gravity_blobs(size=(20, 20), seed=10),
         potential=lambda: ic.smooth_perturbation((20, 20), seed=11, amp=.5).reshape(-1)),
]


def cfg_of(case):
    return _abi.make_config(**case["cfg"])


def fixture_path(name):
    return os.path.join(HERE, name + ".npz")


def main():
    import pyoracle
    pyoracle.build_refcl(quiet=False)
    manifest = {}
    for case in CASES:
        cfg = cfg_of(case)
        init = np.ascontiguousarray(case["init"]()).reshape(-1)
        dtype = init.dtype
        pot = case["potential"]().astype(dtype) if "potential" in case else None
        r = pyoracle.Refcl(cfg)
        r.set_state(init, pot)
        dts = []
        for _ in range(case["steps"]):
            dts.append(r.update(1))
        out = r.get_state()
        meta = dict(case["cfg"])
        meta["steps"] = case["steps"]
        extra = {}
        if pot is not None:
            extra["potential"] = pot
        if pot is not None or case["cfg"].get("use_gravity"):
            extra["final_potential"] = r.get_potential()
        np.savez_compressed(fixture_path(case["name"]), init=init, final=out, dts=np.array(dts),
                            meta=json.dumps(meta), **extra)
        with open(fixture_path(case["name"]), "rb") as f:
            manifest[case["name"]] = hashlib.sha256(f.read()).hexdigest()
        print(case["name"], "dt[-1]=%r" % dts[-1])
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py (refcl: the reference kernels on the CPU)",
                   "sha256": manifest}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
