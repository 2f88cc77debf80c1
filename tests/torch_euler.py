"""Pure-torch FP64 restatement of one EulerRoe step, for gradient checks.

Test infrastructure only: an independent, differentiable (torch autograd) statement
of the scheme the CUDA kernels implement -- ghost fill (res/Euler.cl boundary
kernels), Roe eigenbasis of u^n frozen for the step (res/EulerRoe.cl:51-226),
Delta-q-tilde (res/Roe.cl:152-168), limited flux (res/Roe.cl:170-320), flux
divergence (res/CalcFluxDeriv.cl:7-44) and the Runge-Kutta tableaus in Shu-Osher
form (include/HydroGPU/Integrator/RungeKutta.h, read from the kernel header here so
both use one table).  Matrices are built densely from the textbook formulas; the
operation order is torch's, so results agree with the kernels to rounding, not bits.
Works for 1, 2 and 3 dimensions on arrays shaped (S_z, S_y, S_x, N)[-dim-1:]."""
import os
import re

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
HDR = os.path.join(HERE, "..", "hydrodynamicsgpu_gb300", "csrc", "kernels", "combine_cells.cuh")
INTEGRATOR_INDEX = {"ForwardEuler": 0, "RungeKutta2": 1, "RungeKutta2Heun": 2, "RungeKutta2Ralston": 3,
                    "RungeKutta3": 4, "RungeKutta4": 5, "RungeKutta4_3_8thsRule": 6, "RungeKutta2TVD": 7,
                    "RungeKutta2NonTVD": 8, "RungeKutta3TVD": 9, "RungeKutta4TVD": 10, "RungeKutta4NonTVD": 11}


def _table(name):
    text = open(HDR).read()
    m = re.search(r"#define %s\s*\\\n(.*?)(?:\n\s*#define|\n\s*\n)" % name, text, re.S)
    body = m.group(1).replace("\\\n", " ").replace("{", "[").replace("}", "]")
    return eval(body)


TABLE_A, TABLE_B = _table("HGPU_TABLE_A"), _table("HGPU_TABLE_B")


def tableau(integrator):
    i = INTEGRATOR_INDEX[integrator]
    return TABLE_A[i], TABLE_B[i]


def _mn(a, b):
    """fmin as the kernels and the oracle evaluate it: a NaN operand yields the other
    one, ties yield the second; the derivative is that of the operand selected."""
    return torch.where(torch.isnan(b), a, torch.where(torch.isnan(a), b, torch.where(a < b, a, b)))


def _mx(a, b):
    return torch.where(torch.isnan(b), a, torch.where(torch.isnan(a), b, torch.where(a > b, a, b)))


def _limiter(name, r):
    z = torch.zeros_like(r)
    one = torch.ones_like(r)
    mn, mx = _mn, _mx
    if name == "DonorCell":
        return z
    if name == "LaxWendroff":
        return one
    if name == "BeamWarming":
        return r
    if name == "Fromm":
        return .5 * (1 + r)
    if name == "MinMod":
        return mx(z, mn(r, one))
    if name == "Superbee":
        return mx(z, mx(mn(one, 2 * r), mn(2 * one, r)))
    if name == "VanLeer":
        return mx(z, r) * 2 / (1 + r)
    if name == "MonotizedCentral":
        return mx(z, mn(2 * one, mn(.5 * (1 + r), 2 * r)))
    if name == "VanAlbada1":
        return (r * r + r) / (r * r + 1)
    if name == "Koren":
        return mx(z, mn(2 * r, mn((1 + 2 * r) / 3, 2 * one)))
    raise ValueError("limiter %s not restated" % name)


def _tdim(dim, axis):
    return dim - 1 - axis          # tensor dimension of grid axis `axis` (x = 0)


def ghost_fill(u, dim, methods):
    """methods[axis] = (min, max) with 0 periodic, 1 mirror, 2 free flow, -1 none."""
    N = dim + 2
    for axis in range(dim):
        td = _tdim(dim, axis)
        S = u.shape[td]
        src = list(range(S))
        sign = torch.ones(S, N, dtype=u.dtype)
        for side, m in enumerate(methods[axis]):
            if m < 0:
                continue
            if m == 0:
                pairs = [(0, S - 4), (1, S - 3)] if side == 0 else [(S - 2, 2), (S - 1, 3)]
            elif m == 1:
                pairs = [(0, 3), (1, 2)] if side == 0 else [(S - 1, S - 4), (S - 2, S - 3)]
            else:
                pairs = [(0, 2), (1, 2)] if side == 0 else [(S - 2, S - 3), (S - 1, S - 3)]
            for dst, s in pairs:
                src[dst] = s
                if m == 1:
                    sign[dst, 1 + axis] = -1.
        idx = torch.tensor(src)
        u = torch.index_select(u, td, idx)
        shape = [1] * (dim + 1)
        shape[td] = S
        shape[-1] = N
        u = u * sign.reshape(shape)
    return u


def _perm(side, j):
    return 1 + side if j == 1 else (1 if j == 1 + side else j)


def eigen(uL, uR, gamma, dim, side):
    """lambda (..., N), L and R (..., N, N) in the global frame, for faces between uL and uR."""
    N = dim + 2
    gm1 = gamma - 1

    def prim(u):
        rho = u[..., 0]
        v = u[..., 1:1 + dim] / rho[..., None]
        vv = (v * v).sum(-1)
        eT = u[..., dim + 1] / rho
        p = gm1 * rho * (eT - .5 * vv)
        return v, eT + p / rho, torch.sqrt(rho)

    vL, hL, wL = prim(uL)
    vR, hR, wR = prim(uR)
    nrm = 1 / (wL + wR)
    v = (wL[..., None] * vL + wR[..., None] * vR) * nrm[..., None]
    H = (wL * hL + wR * hR) * nrm
    vv = (v * v).sum(-1)
    c = torch.sqrt((H - .5 * vv) * gm1)
    # normal frame: momentum components swapped 1 <-> 1+side, so tangent t is velocity perm(2+t)-1
    vx = v[..., side]
    vt = [v[..., _perm(side, 2 + t) - 1] for t in range(dim - 1)]
    one = torch.ones_like(vx)
    zero = torch.zeros_like(vx)
    E = N - 1
    # R columns (normal frame): 0, 1, tangents, E
    Rn = [[None] * N for _ in range(N)]
    col0 = [one, vx - c] + vt + [H - c * vx]
    col1 = [one, vx] + vt + [.5 * vv]
    colE = [one, vx + c] + vt + [H + c * vx]
    for i in range(N):
        Rn[i][0], Rn[i][1], Rn[i][E] = col0[i], col1[i], colE[i]
    for t in range(dim - 1):
        for i in range(N):
            Rn[i][2 + t] = one if i == 2 + t else (vt[t] if i == E else zero)
    idd = .5 / (c * c)
    hv = .5 * gm1 * vv
    Ln = [[None] * N for _ in range(N)]
    Ln[0] = [(hv + c * vx) * idd, -(c + gm1 * vx) * idd] + [-gm1 * x * idd for x in vt] + [gm1 * idd]
    Ln[1] = [1 - gm1 * vv * idd, 2 * gm1 * vx * idd] + [2 * gm1 * x * idd for x in vt] + [-2 * gm1 * idd]
    for t in range(dim - 1):
        Ln[2 + t] = [-vt[t]] + [one if j == 2 + t else zero for j in range(1, N)]
    Ln[E] = [(hv - c * vx) * idd, (c - gm1 * vx) * idd] + [-gm1 * x * idd for x in vt] + [gm1 * idd]
    # global frame: L[i][j] = Ln[i][perm(j)], R[g][j] = Rn[perm(g)][j]
    L = torch.stack([torch.stack([Ln[i][_perm(side, j)] for j in range(N)], -1) for i in range(N)], -2)
    R = torch.stack([torch.stack([Rn[_perm(side, g)][j] for j in range(N)], -1) for g in range(N)], -2)
    lam = torch.stack([vx - c] + [vx] * (N - 2) + [vx + c], -1)
    return lam, L, R


def _shift(x, td, k):
    return torch.roll(x, shifts=k, dims=td)


def _face_mask(shape, dim, side):
    """faces along `side` in [2, S-2], transverse [2, S-3] (the kernels' flux faces)."""
    m = torch.ones(shape[:-1], dtype=torch.bool)
    for a in range(dim):
        td = _tdim(dim, a)
        S = shape[td]
        idx = torch.arange(S)
        ok = (idx >= 2) & (idx <= (S - 2 if a == side else S - 3))
        sh = [1] * dim
        sh[td] = S
        m = m & ok.reshape(sh)
    return m


def _interior(shape, dim):
    m = torch.ones(shape[:-1], dtype=torch.bool)
    for a in range(dim):
        td = _tdim(dim, a)
        S = shape[td]
        idx = torch.arange(S)
        sh = [1] * dim
        sh[td] = S
        m = m & ((idx >= 2) & (idx <= S - 3)).reshape(sh)
    return m


def derivative(u, basis, dim, dx, dt, limiter):
    """dU/dt of stage state u with the frozen per-axis basis (lam, L, R on every cell
    index f = the face between f-1 and f)."""
    N = dim + 2
    d = torch.zeros_like(u)
    for side in range(dim):
        td = _tdim(dim, side)
        lam, L, R = basis[side]
        mask = _face_mask(u.shape, dim, side)[..., None]
        uL = _shift(u, td, 1)
        dq = torch.einsum("...ij,...j->...i", L, u - uL)
        dq = torch.where(mask, dq, torch.zeros_like(dq))
        dqM, dqP = _shift(dq, td, 1), _shift(dq, td, -1)
        avg = .5 * (u + uL)
        ft = lam * torch.einsum("...ij,...j->...i", L, avg)
        up = lam >= 0
        theta = torch.where(up, torch.ones_like(lam), -torch.ones_like(lam))
        # r = dq_upwind / dq; where dq == 0 the value (+-Inf or NaN) selects the limiter
        # branch and carries no derivative
        zero = dq == 0
        safe = torch.where(mask & ~zero, dq, torch.ones_like(dq))
        dqUp = torch.where(up, dqM, dqP)
        r = torch.where(zero, (dqUp / dq).detach(), dqUp / safe)
        # limiter of non-finite r: value only (no derivative leaks through masked faces)
        fin = torch.isfinite(r)
        phi = torch.where(fin, _limiter(limiter, torch.where(fin, r, torch.zeros_like(r))),
                          _limiter(limiter, r).detach())
        phi = torch.where(mask, phi, torch.zeros_like(phi))   # unused there; keeps 0 * NaN out of R's cotangent
        eps = lam * (dt / dx[side])
        ft = ft - .5 * lam * dq * (theta + phi * (eps - theta))
        F = torch.einsum("...ij,...j->...i", R, ft)
        F = torch.where(mask, F, torch.zeros_like(F))
        d = d - (_shift(F, td, -1) - F) / dx[side]
    return torch.where(_interior(u.shape, dim)[..., None], d, torch.zeros_like(d))


def step(u, dim, dx, gamma, dt, limiter, integrator, methods):
    """One EulerRoe step with frozen dt (u shaped like the grid, N last)."""
    u0 = ghost_fill(u, dim, methods)
    basis = []
    for side in range(dim):
        td = _tdim(dim, side)
        lam, L, R = eigen(_shift(u0, td, 1), u0, gamma, dim, side)
        basis.append((lam, L, R))
    A, B = tableau(integrator)
    us, ds = [u0], []
    for m in range(len(A)):
        ds.append(derivative(us[-1], basis, dim, dx, dt, limiter))
        nxt = sum(A[m][k] * us[k] + (B[m][k] * dt) * ds[k] for k in range(m + 1))
        us.append(nxt)
    out = us[-1]
    if integrator == "ForwardEuler":
        out = ghost_fill(out, dim, methods)
    return out
