"""Shared inputs for the parity tests: seeded random states and the benchmark ICs."""
import numpy as np

from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

SMALL = {1: (40,), 2: (20, 18), 3: (10, 9, 8)}


def random_state(cfg, seed=0, blocky=False):
    """Positive density/pressure, |v| < .5.  `blocky` quantises the fields so that
    neighbouring cells are often equal (Delta-q-tilde == 0, limiter ratio 0/0 or x/0)."""
    dim = _abi.config_dim(cfg)
    shape = tuple(reversed([cfg.size[i] for i in range(3)]))
    rng = np.random.default_rng(seed)
    rho = rng.uniform(.5, 2., shape)
    p = rng.uniform(.5, 2., shape)
    v = [rng.uniform(-.5, .5, shape) for _ in range(3)]
    if blocky:
        rho = np.round(rho * 2) / 2
        p = np.round(p * 2) / 2
        v = [np.round(x * 4) / 4 for x in v]
    st = ic.build_state_euler(dim, 1.4, rho, v[0], v[1], v[2], p)
    if cfg.precision == _abi.FP32:
        st = st.astype(np.float32)
    return st.reshape(-1)


def same(a, b):
    """Bit-identical up to the sign of zero, NaN == NaN."""
    return np.array_equal(a, b, equal_nan=True)


def canonical(a):
    """A copy of `a` under the parity rule's equivalence: -0 mapped to +0 and every NaN
    to the one quiet-NaN pattern, so that equal states under `same` give equal bytes."""
    c = np.array(a, copy=True)
    c[c == 0] = 0
    c[np.isnan(c)] = np.nan
    return c


def state_digest(a):
    """SHA-256 of the canonical bytes of a state (little-endian, native element type)."""
    import hashlib
    c = canonical(np.asarray(a).reshape(-1))
    return hashlib.sha256(c.astype(c.dtype.newbyteorder("<"), copy=False).tobytes()).hexdigest()


def describe_diff(a, b):
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    bad = ~((a64 == b64) | (np.isnan(a64) & np.isnan(b64)))
    idx = np.flatnonzero(bad)
    if idx.size == 0:
        return "identical"
    d = np.abs(a64[idx] - b64[idx])
    return "%d differing elements, first at %d (%r vs %r), max |diff| %g" % (
        idx.size, idx[0], a64[idx[0]], b64[idx[0]], np.nanmax(d) if np.any(np.isfinite(d)) else float("nan"))


def normwise_rel(a, b, n_states):
    """max over states of max|a-b| / max|b| (the FP32 tolerance measure)."""
    a = a.astype(np.float64).reshape(-1, n_states)
    b = b.astype(np.float64).reshape(-1, n_states)
    out = 0.0
    for j in range(n_states):
        scale = np.max(np.abs(b[:, j]))
        if scale == 0:
            scale = 1.0
        out = max(out, float(np.max(np.abs(a[:, j] - b[:, j]))) / scale)
    return out
