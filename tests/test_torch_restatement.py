"""The pure-torch restatement used for the gradient checks agrees with the oracle.

Independent of the GPU: one step of tests/torch_euler.py with the oracle's CFL dt
against the oracle's step, to rounding (the operation orders differ)."""
import itertools

import numpy as np
import pytest

from _cases import SMALL, random_state
from hydrodynamicsgpu_gb300 import _abi

torch = pytest.importorskip("torch")
import torch_euler as te  # noqa: E402


def grid_shape(cfg):
    dim = _abi.config_dim(cfg)
    return tuple(reversed([cfg.size[i] for i in range(dim)])) + (dim + 2,)


def methods_of(cfg, dim):
    return [(cfg.boundary[a][0], cfg.boundary[a][1]) for a in range(dim)]


@pytest.mark.parametrize("dim,bnd,integ,lim", [
    (1, "FREEFLOW", "ForwardEuler", "Superbee"),
    (1, "PERIODIC", "RungeKutta4", "MinMod"),
    (2, "PERIODIC", "RungeKutta2", "MinMod"),
    (2, "PERIODIC", "RungeKutta3TVD", "VanLeer"),
    (2, "MIRROR", "RungeKutta3TVD", "Superbee"),
    (2, "FREEFLOW", "RungeKutta2Heun", "MonotizedCentral"),
    (3, "MIRROR", "RungeKutta2", "Superbee"),
])
def test_torch_step_matches_oracle(oracle_mod, dim, bnd, integ, lim):
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[dim], boundary=bnd, limiter=lim, integrator=integ)
    u = random_state(cfg, seed=7)
    o = oracle_mod.Oracle(cfg)
    o.set_state(u)
    dt = o.update(1)
    ref = o.get_state()
    _, dx, gamma, _ = oracle_mod.resolve(cfg)
    out = te.step(torch.tensor(u.reshape(grid_shape(cfg))), dim, dx, gamma, dt, lim, integ, methods_of(cfg, dim))
    out = out.reshape(-1).numpy()
    assert np.all(np.isfinite(ref))
    assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref))
