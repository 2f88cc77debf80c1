"""Golden fixtures produced by the reference's own kernels (tests/golden/make_golden.py).

CPU: the oracle restatement must reproduce every fixture bit for bit (dt of every
step and the final state, NaN == NaN).  GPU: so must the CUDA path, through the C ABI.
"""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

from _cases import describe_diff, same
from hydrodynamicsgpu_gb300 import _abi

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(HERE, "*.npz")))
NAMES = [os.path.basename(f)[:-4] for f in FIXTURES]


def load(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    steps = meta.pop("steps")
    cfg = _abi.make_config(**meta)
    return cfg, d["init"], d["final"], d["dts"], steps


def potentials(name):
    """(input potential channel or None, final potential or None) of a fixture."""
    d = np.load(os.path.join(HERE, name + ".npz"))
    return (d["potential"] if "potential" in d.files else None,
            d["final_potential"] if "final_potential" in d.files else None)


def test_manifest_hashes():
    with open(os.path.join(HERE, "MANIFEST.json")) as f:
        man = json.load(f)["sha256"]
    assert sorted(man) == NAMES
    for name in NAMES:
        with open(os.path.join(HERE, name + ".npz"), "rb") as f:
            assert hashlib.sha256(f.read()).hexdigest() == man[name], name


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_golden(oracle_mod, name):
    cfg, init, final, dts, steps = load(name)
    pot, final_pot = potentials(name)
    o = oracle_mod.Oracle(cfg)
    o.set_state(init, pot)
    for k in range(steps):
        assert o.update(1) == dts[k], "%s: dt of step %d" % (name, k)
    out = o.get_state()
    assert same(out, final), "%s: %s" % (name, describe_diff(out, final))
    if final_pot is not None:
        assert same(o.get_potential(), final_pot), name


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_golden(hg, name):
    cfg, init, final, dts, steps = load(name)
    pot, final_pot = potentials(name)
    s = hg.Solver(cfg)
    s.resetState(init, pot)
    for k in range(steps):
        dt = s.update(1)
        if cfg.precision == _abi.FP64:
            assert dt == dts[k], "%s: dt of step %d: %r vs %r" % (name, k, dt, dts[k])
    out = s.getState()
    out_pot = s.getPotential()
    s.close()
    if cfg.precision == _abi.FP64:
        assert same(out, final), "%s: %s" % (name, describe_diff(out, final))
        if final_pot is not None:
            assert same(out_pot, final_pot), name
    else:
        from _cases import normwise_rel
        assert normwise_rel(out, final, _abi.config_dim(cfg) + 2) <= 1e-5
        if final_pot is not None:
            assert normwise_rel(out_pot, final_pot, 1) <= 1e-5
