"""Output: the display scalar (convertToTex) and Solver::save's FITS files.

The display scalar of every cell must equal the oracle's bit for bit (the oracle's
restatement is pinned to the reference's own convertToTex in test_oracle_pin.py);
the saved FITS images must hold the state channels as 32-bit floats."""
import itertools
import os

import numpy as np
import pytest

from _cases import SMALL, random_state
from hydrodynamicsgpu_gb300 import _abi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("solver,dim,prec", list(itertools.product(["EulerRoe", "EulerHLLC", "EulerHLL"], [1, 2, 3],
                                                                   [_abi.FP64, _abi.FP32])))
def test_display_matches_oracle(hg, oracle_mod, solver, dim, prec):
    cfg = _abi.make_config(solver=solver, size=SMALL[dim], boundary="MIRROR", integrator="RungeKutta2",
                           precision=prec)
    init = random_state(cfg, seed=40 + dim)
    s, o = hg.Solver(cfg), oracle_mod.Oracle(cfg)
    s.resetState(init)
    o.set_state(init)
    s.update(2)
    o.update(2)
    for m, name in enumerate(_abi.display_names(dim)):
        a = s.display(name).reshape(-1)
        b = o.display(m)
        assert np.array_equal(a, b, equal_nan=True), name
    with pytest.raises(hg.HgpuError):
        s.display(7 + dim)
    s.close()


def read_fits(path):
    """Minimal FITS reader: primary HDU, BITPIX -32, returns (header dict, float32 array)."""
    raw = open(path, "rb").read()
    hdr, pos = {}, 0
    while True:
        block = raw[pos:pos + 2880]
        pos += 2880
        done = False
        for k in range(36):
            card = block[80 * k:80 * (k + 1)].decode("ascii")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] == "= ":
                hdr[key] = card[10:].strip()
        if done:
            break
    shape = tuple(int(hdr["NAXIS%d" % i]) for i in range(int(hdr["NAXIS"]), 0, -1))
    n = int(np.prod(shape))
    data = np.frombuffer(raw[pos:pos + 4 * n], dtype=">f4").reshape(shape)
    assert len(raw) % 2880 == 0
    return hdr, data


@pytest.mark.parametrize("dim,prec", [(1, _abi.FP64), (2, _abi.FP64), (3, _abi.FP32)])
def test_save_fits(hg, tmp_path, dim, prec):
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[dim], boundary="PERIODIC", integrator="RungeKutta2",
                           precision=prec)
    s = hg.Solver(cfg)
    s.resetState(random_state(cfg, seed=5))
    s.update(1)
    assert s.save(str(tmp_path)) == 0
    assert s.save(str(tmp_path)) == 1                       # the next free index
    st = s.getState().reshape(s.shape())
    names = ["DENSITY", "MOMENTUM_X", "MOMENTUM_Y", "MOMENTUM_Z"][:1 + dim] + ["ENERGY_TOTAL"]
    for j, n in enumerate(names):
        hdr, data = read_fits(os.path.join(str(tmp_path), "%s1.fits" % n))
        assert hdr["BITPIX"] == "-32" and int(hdr["NAXIS1"]) == cfg.size[0]
        assert np.array_equal(data.astype(np.float32), st[..., j].astype(np.float32))
    _, pot = read_fits(os.path.join(str(tmp_path), "potential0.fits"))
    assert not pot.any()
    s.close()
