"""Initial conditions: the Euler entries of the reference's IC catalogue, vectorised.

The reference evaluates a Lua ``initState(x, y, z)`` at every cell centre of the
full grid, ghosts included (src/Solver/Solver.cpp:357-382), with
    pos = (xmax - xmin) * (i + .5) / size + xmin
and builds the conserved state with ``buildStateEuler`` (res/util.lua:36-80):
    E = rho * (.5 * (vx*vx + vy*vy + vz*vz) + p / ((gamma - 1) * rho))
mapped to the N solver states by Euler::readStateCell (src/Equation/Euler.cpp:78-89).
The potential channel is zero (useGravity = false), so nothing is added to E
(src/Solver/SelfGravitation.cpp:89-94).

Inputs that the reference draws from Lua's math.random are drawn here from seeded
numpy generators, so they are reproducible; the workload shapes and value ranges
follow the benchmark configurations.
"""
import math

import numpy as np


def cell_centers(size, xmin, xmax):
    """Per-axis cell-centre coordinates (Solver.cpp:364), ghosts included."""
    out = []
    for i in range(3):
        n = int(size[i]) if i < len(size) else 1
        lo = float(xmin[i]) if i < len(xmin) else -.5
        hi = float(xmax[i]) if i < len(xmax) else .5
        idx = np.arange(n, dtype=np.float64)
        out.append((hi - lo) * (idx + .5) / float(n) + lo)
    return out


def mesh(size, xmin, xmax):
    cx, cy, cz = cell_centers(size, xmin, xmax)
    z, y, x = np.meshgrid(cz, cy, cx, indexing="ij")  # C order (z, y, x): x fastest
    return x, y, z


def build_state_euler(dim, gamma, density, vx, vy=0.0, vz=0.0, pressure=1.0, dtype=np.float64):
    """res/util.lua:36-80 followed by Euler::readStateCell; returns AoS (..., N)."""
    density = np.asarray(density, dtype=np.float64)
    shape = density.shape
    vx = np.broadcast_to(np.asarray(vx, dtype=np.float64), shape)
    vy = np.broadcast_to(np.asarray(vy if dim > 1 else 0.0, dtype=np.float64), shape)
    vz = np.broadcast_to(np.asarray(vz if dim > 2 else 0.0, dtype=np.float64), shape)
    pressure = np.broadcast_to(np.asarray(pressure, dtype=np.float64), shape)
    ek = .5 * (vx * vx + vy * vy + vz * vz)
    ei = pressure / ((gamma - 1) * density)
    e_total = density * (ek + ei)
    comps = [density, density * vx]
    if dim > 1:
        comps.append(density * vy)
    if dim > 2:
        comps.append(density * vz)
    comps.append(e_total)
    return np.stack(comps, axis=-1).astype(dtype)


def flat(state):
    return np.ascontiguousarray(state).reshape(-1)


def sod(size=(1024,), xmin=(0.,), xmax=(1.,), gamma=1.4, x0=.5, dtype=np.float64):
    """Sod shock tube (res/initConds.lua:62-79, shifted so the diaphragm sits at x0):
    (rho, u, p) = (1, 0, 1) left of x0, (0.125, 0, 0.1) right."""
    dim = len([s for s in size if s > 1])
    x, y, z = mesh(size, xmin, xmax)
    inside = x < x0
    rho = np.where(inside, 1.0, .125)
    p = np.where(inside, 1.0, .1)
    return build_state_euler(dim, gamma, rho, 0.0, 0.0, 0.0, p, dtype)


def kelvin_helmholtz(size=(2048, 2048), xmin=(-.5, -.5), xmax=(.5, .5), gamma=1.4, seed=0,
                     noise=1e-3, amp=.01, dtype=np.float64):
    """Shear layer of the 2D benchmark: rho=2, u=+0.5 for |y|<0.25, else rho=1, u=-0.5;
    p=2.5; v = amp*sin(4*pi*x) plus seeded uniform noise of amplitude `noise` on u and v.
    (The reference's own Kelvin-Helmholtz entry, res/initConds.lua:303-326, is
    `kelvin_helmholtz_reference`.)"""
    dim = 2
    x, y, z = mesh(size, xmin, xmax)
    rng = np.random.default_rng(seed)
    inside = np.abs(y) < .25
    rho = np.where(inside, 2.0, 1.0)
    u = np.where(inside, .5, -.5) + rng.uniform(-noise, noise, size=x.shape)
    v = amp * np.sin(4 * math.pi * x) + rng.uniform(-noise, noise, size=x.shape)
    return build_state_euler(dim, gamma, rho, u, v, 0.0, 2.5, dtype)


def kelvin_helmholtz_reference(size=(256, 256), xmin=(-.5, -.5, -.5), xmax=(.5, .5, .5), gamma=1.4,
                               dtype=np.float64):
    """res/initConds.lua:303-326 verbatim in numpy: noise = size[1] * 2e-5,
    theta = (x - xmin)/(xmax - xmin) * 2 pi (times (z-zmin)/(zmax-zmin) in 3D)."""
    dim = len([s for s in size if s > 1])
    x, y, z = mesh(size, xmin, xmax)
    inside = (y > -.25) & (y < .25)
    theta = (x - xmin[0]) / (xmax[0] - xmin[0]) * 2 * math.pi
    if dim >= 3:
        theta = theta * (z - xmin[2]) / (xmax[2] - xmin[2])
    noise = size[0] * 2e-5
    rho = np.where(inside, 2.0, 1.0)
    vx = np.cos(theta) * noise + np.where(inside, -.5, .5)
    vy = np.sin(theta) * noise
    vz = np.sin(theta) * noise
    return build_state_euler(dim, gamma, rho, vx, vy, vz, 2.5, dtype)


def quadrant(size, q, xmin=(-.5, -.5), xmax=(.5, .5), gamma=1.4, dtype=np.float64):
    """Four-quadrant Riemann problem (buildStateEulerQuadrant, res/util.lua:82-96):
    y > 0: x > 0 -> q1 else q2;  y <= 0: x < 0 -> q3 else q4.
    Each q is (rho, u, v, p)."""
    x, y, z = mesh(size, xmin, xmax)
    sel = np.where(y > 0, np.where(x > 0, 0, 1), np.where(x < 0, 2, 3))
    qa = np.asarray(q, dtype=np.float64)
    rho, u, v, p = (qa[sel, k] for k in range(4))
    return build_state_euler(2, gamma, rho, u, v, 0.0, p, dtype)


# res/initConds.lua:84-187 (Configurations 1-6 of Kurganov & Tadmor's catalogue)
CONFIGURATIONS = {
    1: [(1, 0, 0, 1), (.5197, -.7259, 0, .4), (.1072, -.7259, -1.4045, .0439), (.2579, 0, -1.4045, .15)],
    2: [(1, 0, 0, 1), (.5197, -.7259, 0, .4), (1, -.7259, -.7259, 1), (.5197, 0, -.7259, .4)],
    3: [(1.5, 0, 0, 1.5), (.5323, 1.206, 0, .3), (.138, 1.206, 1.206, .029), (.5323, 0, 1.206, .3)],
    4: [(1.1, 0, 0, 1.1), (.5065, .8939, 0, .35), (1.1, .8939, .8939, 1.1), (.5065, 0, .8939, .35)],
    5: [(1, -.75, -.5, 1), (2, -.75, .5, 1), (1, .75, .5, 1), (3, .75, -.5, 1)],
    6: [(1, .75, -.5, 1), (2, .75, .5, 1), (1, -.75, .5, 1), (3, -.75, -.5, 1)],
}


def configuration(n, size=(256, 256), gamma=1.4, dtype=np.float64):
    return quadrant(size, CONFIGURATIONS[n], gamma=gamma, dtype=dtype)


def _exp_basic(x):
    """exp(x) from basic IEEE operations only (add, multiply, divide, scaling by 2^n), so
    that the same inputs give the same bits on every platform (libm and vectorised
    numpy exponentials differ between machines in the last bit).  Cody-Waite range
    reduction x = n ln2 + r, |r| <= ln2 / 2, with ln2 split into a 32-bit head and a
    tail, then the Taylor series of exp(r) to degree 18 by Horner's rule (truncation
    below 1e-22 relative), scaled by 2^n."""
    x = np.asarray(x, dtype=np.float64)
    ln2_hi = 0.693147180369123816490     # ln 2 rounded to 32 significant bits
    ln2_lo = 1.90821492927058770002e-10  # ln 2 - ln2_hi
    n = np.rint(x / 0.6931471805599453)
    r = (x - n * ln2_hi) - n * ln2_lo
    p = np.ones_like(r)
    for k in range(18, 0, -1):
        p = 1.0 + p * r / float(k)
    return np.ldexp(p, n.astype(np.int64))


def _box_periodic(a, axis, width):
    """Periodic moving average of odd `width` along `axis`: the first window summed
    term by term, each next one by adding the entering and subtracting the leaving
    plane, in a fixed order."""
    h = width // 2
    b = np.moveaxis(a, axis, 0)
    n = b.shape[0]
    out = np.empty_like(b)
    acc = np.zeros_like(b[0])
    for k in range(-h, h + 1):
        acc = acc + b[k % n]
    out[0] = acc
    for i in range(1, n):
        acc = (acc + b[(i + h) % n]) - b[(i - 1 - h) % n]
        out[i] = acc
    return np.moveaxis(out / float(width), 0, axis)


def _fsum(a):
    """Exactly rounded sum of an array (math.fsum over chunks of partial sums is not
    exact, so the values themselves are passed)."""
    return math.fsum(np.ravel(a).tolist())


def lognormal_grf(size=(256, 256, 256), xmin=(0., 0., 0.), xmax=(1., 1., 1.), gamma=5. / 3., sigma=.5,
                  corr_cells=16.0, seed=1, dtype=np.float64):
    """3D benchmark: density exp(sigma*G) normalised to mean 1, where G is a
    unit-variance Gaussian random field with a correlation length of `corr_cells`
    cells; p=1, u=0.  G is seeded white noise (uniform, unit variance) smoothed on the
    periodic grid by three passes of a moving average per axis, whose product is a
    near-Gaussian kernel of standard deviation sqrt((w^2 - 1)/4) ~ corr_cells cells
    (w odd), then centred and scaled to unit variance with exactly rounded sums.
    Only basic IEEE operations in a fixed order are used (see _exp_basic), so a seed
    gives the same state, bit for bit, on every platform."""
    nz, ny, nx = size[2], size[1], size[0]
    rng = np.random.default_rng(seed)
    s3 = math.sqrt(3.0)
    g = rng.uniform(-s3, s3, (nz, ny, nx))
    width = int(round(math.sqrt(4. * corr_cells * corr_cells + 1.)))
    width += 1 - width % 2
    for axis in (0, 1, 2):
        for _ in range(3):
            g = _box_periodic(g, axis, width)
    count = float(g.size)
    g = g - _fsum(g) / count
    g = g / math.sqrt(_fsum(g * g) / count)
    rho = _exp_basic(sigma * g)
    rho = rho / (_fsum(rho) / count)
    return build_state_euler(3, gamma, rho, 0.0, 0.0, 0.0, 1.0, dtype)


def random_quadrant_problems(n=512, seed=2, lo=32, hi=512):
    """Batched sweep inputs: side = 16*round(exp(U(ln lo, ln hi))/16); per quadrant
    rho, p ~ U[0.1, 2], u, v ~ U[-1, 1]; boundary periodic or free-flow per problem.
    Returns a list of dicts (side, quadrants, boundary)."""
    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(n):
        side = int(16 * round(math.exp(rng.uniform(math.log(lo), math.log(hi))) / 16))
        side = max(side, 16)
        q = []
        for _k in range(4):
            rho = rng.uniform(.1, 2.)
            u = rng.uniform(-1., 1.)
            v = rng.uniform(-1., 1.)
            p = rng.uniform(.1, 2.)
            q.append((rho, u, v, p))
        boundary = "PERIODIC" if rng.uniform() < .5 else "FREEFLOW"
        probs.append({"side": side, "quadrants": q, "boundary": boundary})
    return probs


def smooth_perturbation(size, seed=200, amp=1e-2, modes=4):
    """Seeded smooth periodic perturbation field (sum of a few low Fourier modes)."""
    x, y, z = mesh(size, (-.5, -.5, -.5), (.5, .5, .5))
    rng = np.random.default_rng(seed)
    f = np.zeros_like(x)
    for _ in range(modes):
        kx, ky = rng.integers(1, 4, size=2)
        ph = rng.uniform(0, 2 * math.pi)
        f += np.sin(2 * math.pi * (kx * x + ky * y) + ph)
    return amp * f / modes


def gravity_blobs(size=(64, 64), xmin=(-.5, -.5, -.5), xmax=(.5, .5, .5), gamma=1.4, nblobs=3, seed=7,
                  pressure=10.0, dtype=np.float64):
    """Self-gravity workload: uniform background density 1 plus `nblobs` Gaussian
    over-densities (seeded centres in the inner half of the domain, amplitudes
    U(1, 3), widths U(.05, .12) of the box), at rest, uniform pressure.  The
    pressure is high enough that the internal energy stays positive after the
    reference's reset adds the potential's starting guess (-density) to the total
    energy."""
    dim = len([s for s in size if s > 1])
    x, y, z = mesh(size, xmin, xmax)
    rng = np.random.default_rng(seed)
    rho = np.ones_like(x)
    for _ in range(nblobs):
        c = rng.uniform(-.25, .25, 3)
        a = rng.uniform(1., 3.)
        w = rng.uniform(.05, .12)
        r2 = (x - c[0]) ** 2 + (y - c[1]) ** 2 * (dim > 1) + (z - c[2]) ** 2 * (dim > 2)
        rho = rho + a * np.exp(-r2 / (2 * w * w))
    return build_state_euler(dim, gamma, rho, 0.0, 0.0, 0.0, pressure, dtype)
