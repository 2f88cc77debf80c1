"""The benchmark configurations run for their full length, pinned to the reference's
own kernels.

tests/golden/fullsize/*.json hold what refcl (HydroGPU's res/*.cl compiled for the
CPU, driven in Solver::update order, src/Solver/Solver.cpp:521-546) produced for
  * KH 2048^2 EulerRoe RK4 MinMod periodic, 500 steps,
  * KH 2048^2 EulerHLLC RK4 periodic, 500 steps,
  * the 256^3 log-normal EulerHLLC run (TVD-RK2, VanLeer, mirror, gamma 5/3, CFL 0.4),
    200 steps:
every step's dt and the SHA-256 of the state every 50 steps and at the end, in the
parity rule's canonical form (tests/_cases.py state_digest).  The GPU must reproduce
every dt and every digest bit for bit; the recipe is tests/golden/make_fullsize.py.

The FP32 instantiation is checked against the FP32 oracle on the same 2048^2 run
for 100 steps, within 1e-5 normwise per conserved variable.
"""
import json
import os
import sys

import numpy as np
import pytest

from _cases import normwise_rel, state_digest
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = os.path.join(HERE, "golden", "fullsize")
NAMES = ["kh2048_roe_rk4_minmod_periodic", "kh2048_hllc_rk4_periodic", "grf256_hllc_tvdrk2_mirror"]


def load(name):
    path = os.path.join(FIXTURES, name + ".json")
    if not os.path.exists(path):
        pytest.skip("fixture %s not recorded (tests/golden/make_fullsize.py)" % name)
    with open(path) as f:
        return json.load(f)


def make_init(fx):
    kw = {k: tuple(v) if isinstance(v, list) else v for k, v in fx["init"]["kwargs"].items()}
    return np.ascontiguousarray(getattr(ic, fx["init"]["fn"])(**kw)).reshape(-1)


def make_cfg(fx):
    kw = {k: tuple(v) if isinstance(v, list) else v for k, v in fx["cfg"].items()}
    return _abi.make_config(**kw)


@pytest.mark.parametrize("name,fused", [(n, False) for n in NAMES] + [(NAMES[0], True)])
def test_full_length_run_matches_reference_kernels(hg, name, fused):
    """fused: the same run with each Runge-Kutta stage as the two fused per-direction
    kernels (hgpu_set_fused_stages)."""
    fx = load(name)
    init = make_init(fx)
    assert state_digest(init) == fx["init_sha256"], \
        "the initial-condition generator gives a different state on this platform"
    s = hg.Solver(make_cfg(fx))
    try:
        if fused:
            s.set_fused_stages(True)
        s.resetState(init)
        for k in range(1, fx["steps"] + 1):
            dt = s.update(1)
            assert float(dt).hex() == fx["dt_hex"][k - 1], \
                "step %d: dt %s, reference kernels %s" % (k, float(dt).hex(), fx["dt_hex"][k - 1])
            want = fx["state_sha256"].get(str(k))
            if want is not None:
                final = s.getState()
                if state_digest(final) != want:
                    idx = np.array(fx["sample_index"])
                    got = [float(final[i]).hex() for i in idx] if k == fx["steps"] else []
                    bad = [int(i) for i, a, b in zip(idx, got, fx["sample_hex"]) if a != b]
                    pytest.fail("step %d: state differs from the reference kernels' (final samples "
                                "differing: %s)" % (k, bad[:8]))
    finally:
        s.close()


def test_kh_2048_fp32_100_steps_vs_fp32_oracle(hg, oracle_mod):
    """KH 2048^2 EulerRoe RK4 MinMod in FP32 for 100 steps, GPU against the FP32 oracle
    (the C restatement of the reference kernels with real = float), each with its own
    CFL dt: every dt within 1e-5 relative, the final state within 1e-5 normwise per
    conserved variable.  The oracle runs on all host cores."""
    cfg = _abi.make_config(solver="EulerRoe", size=(2048, 2048), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", cfl=.5, precision=_abi.FP32)
    init = ic.kelvin_helmholtz(size=(2048, 2048), seed=0).astype(np.float32).reshape(-1)
    steps = 100
    s = hg.Solver(cfg)
    try:
        s.resetState(init)
        dts = [s.update(1) for _ in range(steps)]
        gpu = s.getState()
    finally:
        s.close()
    oracle_mod.set_threads(os.cpu_count() or 1)
    ref = oracle_mod.Oracle(cfg)
    ref.set_state(init)
    rdts = [ref.update(1) for _ in range(steps)]
    out = ref.get_state()
    worst_dt = max(abs(a - b) / abs(b) for a, b in zip(dts, rdts))
    err = normwise_rel(gpu, out, 4)
    sys.stdout.write("fp32 2048^2 100 steps: dt rel %.3g, state normwise %.3g\n" % (worst_dt, err))
    assert worst_dt <= 1e-5, worst_dt
    assert err <= 1e-5, err
