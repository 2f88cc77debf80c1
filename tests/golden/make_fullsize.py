#!/usr/bin/env python3
"""Record the benchmark configurations' full-length runs from the reference's own kernels.

Each run is driven by "refcl" (HydroGPU's res/*.cl compiled for the CPU by
oracle/refcl/build_refcl.py, stepped in the reference host order of
Solver::update, src/Solver/Solver.cpp:521-546) for the benchmark's full step count.
The states are too large to commit (134 MB for 2048^2, 671 MB for 256^3), so a
fixture keeps what a GPU run can be checked against bit for bit:

  * the SHA-256 of the initial state (the seeded generator's output; a test first
    checks that its own generator reproduces it);
  * the dt of every step, as hexadecimal floats;
  * the SHA-256 of the state every `every` steps and after the last step, in the
    parity rule's canonical form (-0 as +0, one NaN pattern; tests/_cases.py);
  * 64 seeded sample cells of the final state, for diagnosis.

Run from the repository root where oracle/_ref/ can be built (the reference sources
are needed once); each run takes tens of minutes on eight cores:

    python tests/golden/make_fullsize.py [--only NAME] [--threads N]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "fullsize")
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

from hydrodynamicsgpu_gb300 import _abi  # noqa: E402
from hydrodynamicsgpu_gb300 import initconds as ic  # noqa: E402
from _cases import state_digest  # noqa: E402

KH = dict(size=(2048, 2048), boundary="PERIODIC", limiter="MinMod", integrator="RungeKutta4", cfl=.5)
GRF = dict(size=(256, 256, 256), xmin=(0, 0, 0), xmax=(1, 1, 1), gamma=5. / 3., boundary="MIRROR",
           limiter="VanLeer", integrator="RungeKutta2TVD", cfl=.4)

RUNS = [
    dict(name="kh2048_roe_rk4_minmod_periodic", steps=500, every=50,
         cfg=dict(KH, solver="EulerRoe"), init=("kelvin_helmholtz", dict(size=(2048, 2048), seed=0))),
    dict(name="kh2048_hllc_rk4_periodic", steps=500, every=50,
         cfg=dict(KH, solver="EulerHLLC"), init=("kelvin_helmholtz", dict(size=(2048, 2048), seed=0))),
    dict(name="grf256_hllc_tvdrk2_mirror", steps=200, every=50,
         cfg=dict(GRF, solver="EulerHLLC"), init=("lognormal_grf", dict(size=(256, 256, 256), seed=1))),
]
SAMPLES = 64


def make_init(spec):
    fn, kw = spec
    return np.ascontiguousarray(getattr(ic, fn)(**kw)).reshape(-1)


def make_cfg(run):
    return _abi.make_config(**run["cfg"])


def fixture_path(name):
    return os.path.join(OUT, name + ".json")


def load(name):
    with open(fixture_path(name)) as f:
        return json.load(f)


def sample_indices(count, seed=12345):
    return np.sort(np.random.default_rng(seed).choice(count, SAMPLES, replace=False))


def record(run, threads):
    import pyoracle
    cfg = make_cfg(run)
    init = make_init(run["init"])
    r = pyoracle.Refcl(cfg)
    r.set_threads(threads)
    r.set_state(init)
    dts, checkpoints = [], {}
    t0 = time.time()
    for k in range(1, run["steps"] + 1):
        dts.append(r.update(1))
        if k % run["every"] == 0 or k == run["steps"]:
            checkpoints[str(k)] = state_digest(r.get_state())
            print("%s step %d dt %r  %.0f s" % (run["name"], k, dts[-1], time.time() - t0), flush=True)
    final = r.get_state()
    idx = sample_indices(final.size)
    out = dict(
        name=run["name"], generator="refcl: the reference's res/*.cl compiled for the CPU, "
                                    "oracle/refcl/build_refcl.py, driven in Solver::update order",
        cfg=run["cfg"], init=dict(fn=run["init"][0], kwargs=run["init"][1]), init_sha256=state_digest(init),
        steps=run["steps"], every=run["every"], dt_hex=[float(d).hex() for d in dts],
        state_sha256=checkpoints, sample_index=[int(i) for i in idx],
        sample_hex=[float(final[i]).hex() for i in idx], threads=threads, seconds=round(time.time() - t0, 1))
    os.makedirs(OUT, exist_ok=True)
    with open(fixture_path(run["name"]) + ".tmp", "w") as f:
        json.dump(out, f, indent=0)
    os.replace(fixture_path(run["name"]) + ".tmp", fixture_path(run["name"]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", action="append")
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    a = ap.parse_args()
    import pyoracle
    pyoracle.build_refcl(quiet=True)
    for run in RUNS:
        if a.only and run["name"] not in a.only:
            continue
        record(run, a.threads)


if __name__ == "__main__":
    main()
