"""Adjoint of the EulerRoe step (hgpu_adjoint_step, hgpu_checkpoint_*), FP64.

Checked three ways: against the gradient of the pure-torch restatement
(tests/torch_euler.py, autograd; agreement to 1e-10 relative), against central
finite differences of the CUDA forward with dt frozen (eps 1e-6 along unit
random directions, agreement 1e-6 relative), and the checkpointed trajectory against a chain of single-step
products (identical bits for every checkpoint interval)."""
import numpy as np
import pytest

from _cases import SMALL, random_state
from hydrodynamicsgpu_gb300 import _abi
from hydrodynamicsgpu_gb300 import initconds as ic

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import torch_euler as te  # noqa: E402

TORCH_TOL = 1e-10
FD_TOL = 1e-6
FD_EPS = 1e-6


def grid_shape(cfg):
    dim = _abi.config_dim(cfg)
    return tuple(reversed([cfg.size[i] for i in range(dim)])) + (dim + 2,)


def methods_of(cfg, dim):
    return [(cfg.boundary[a][0], cfg.boundary[a][1]) for a in range(dim)]


def cuda(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def cfl_dt(hg, cfg, u):
    s = hg.Solver(cfg)
    try:
        s.resetState(u)
        return s.update(1)
    finally:
        s.close()


def gpu_vjp(hg, cfg, u, lam, dt):
    s = hg.Solver(cfg)
    try:
        du, dl = cuda(u), cuda(lam)
        out = torch.empty_like(du)
        torch.cuda.synchronize()
        s.adjoint_step(du.data_ptr(), dl.data_ptr(), out.data_ptr(), dt)
        s.synchronize()
        return out.cpu().numpy()
    finally:
        s.close()


def gpu_frozen(hg, cfg, u, dts):
    s = hg.Solver(cfg)
    try:
        s.resetState(u)
        s.update_frozen_dt(dts)
        return s.getState().copy()
    finally:
        s.close()


def torch_vjp(oracle_mod, cfg, u, lam, dts):
    dim = _abi.config_dim(cfg)
    _, dx, gamma, _ = oracle_mod.resolve(cfg)
    lim = _abi.LIMITERS[cfg.limiter]
    integ = _abi.INTEGRATORS[cfg.integrator]
    x = torch.tensor(u.reshape(grid_shape(cfg)), requires_grad=True)
    y = x
    for dt in dts:
        y = te.step(y, dim, dx, gamma, dt, lim, integ, methods_of(cfg, dim))
    (y * torch.tensor(lam.reshape(grid_shape(cfg)))).sum().backward()
    return x.grad.reshape(-1).numpy(), y.detach().reshape(-1).numpy()


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


CASES = [
    (1, "FREEFLOW", "ForwardEuler", "Superbee"),
    (1, "PERIODIC", "RungeKutta4", "MinMod"),
    (1, "MIRROR", "RungeKutta2", "MonotizedCentral"),
    (2, "PERIODIC", "RungeKutta2", "MinMod"),
    (2, "PERIODIC", "ForwardEuler", "VanLeer"),
    (2, "MIRROR", "RungeKutta3TVD", "Superbee"),
    (2, "FREEFLOW", "RungeKutta2Heun", "MonotizedCentral"),
    (2, "PERIODIC", "RungeKutta4", "Koren"),
    (2, [("PERIODIC", "PERIODIC"), ("MIRROR", "FREEFLOW")], "RungeKutta2", "MinMod"),
    (2, "PERIODIC", "RungeKutta2", "VanAlbada1"),
    (3, "MIRROR", "RungeKutta2", "Superbee"),
    (3, "PERIODIC", "RungeKutta4", "MinMod"),
]


@pytest.mark.parametrize("dim,bnd,integ,lim", CASES)
def test_adjoint_step_matches_torch(hg, oracle_mod, dim, bnd, integ, lim):
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[dim], boundary=bnd, limiter=lim, integrator=integ)
    u = random_state(cfg, seed=3 + dim)
    lam = np.random.default_rng(17).standard_normal(u.size)
    dt = cfl_dt(hg, cfg, u)
    g_ref, y_ref = torch_vjp(oracle_mod, cfg, u, lam, [dt])
    y = gpu_frozen(hg, cfg, u, [dt])
    assert rel(y, y_ref) <= 1e-12
    g = gpu_vjp(hg, cfg, u, lam, dt)
    assert rel(g, g_ref) <= TORCH_TOL, rel(g, g_ref)


@pytest.mark.parametrize("dim,bnd,integ,lim", CASES[:6] + CASES[9:])
def test_adjoint_step_matches_finite_differences(hg, dim, bnd, integ, lim):
    cfg = _abi.make_config(solver="EulerRoe", size=SMALL[dim], boundary=bnd, limiter=lim, integrator=integ)
    u = random_state(cfg, seed=30 + dim)
    rng = np.random.default_rng(300)
    lam = rng.standard_normal(u.size)
    dt = cfl_dt(hg, cfg, u)
    g = gpu_vjp(hg, cfg, u, lam, dt)
    for _ in range(4):
        d = rng.standard_normal(u.size)
        d /= np.linalg.norm(d)                # unit direction
        fp = gpu_frozen(hg, cfg, u + FD_EPS * d, [dt])
        fm = gpu_frozen(hg, cfg, u - FD_EPS * d, [dt])
        fd = float(np.dot(lam, fp - fm)) / (2 * FD_EPS)
        ad = float(np.dot(g, d))
        assert abs(fd - ad) <= FD_TOL * abs(ad), (fd, ad)


def test_frozen_dt_step_is_the_cfl_step(hg):
    """update_frozen_dt with the dt update() chose reproduces update() bit for bit."""
    for integ in ["ForwardEuler", "RungeKutta2", "RungeKutta4", "RungeKutta3TVD", "RungeKutta4TVD"]:
        cfg = _abi.make_config(solver="EulerRoe", size=(24, 20), boundary="MIRROR", limiter="Superbee",
                               integrator=integ)
        u = random_state(cfg, seed=5)
        a = hg.Solver(cfg)
        a.resetState(u)
        dts = [a.update(1) for _ in range(4)]
        b = gpu_frozen(hg, cfg, u, dts)
        assert np.array_equal(a.getState(), b, equal_nan=True)
        a.close()


def kh_small(n=24, seed=100, limiter="MinMod"):
    size = (n + 4, n + 4)
    st = ic.kelvin_helmholtz(size=size, seed=seed)
    return _abi.make_config(solver="EulerRoe", size=size, boundary="PERIODIC", limiter=limiter,
                            integrator="RungeKutta2"), st.reshape(-1)


def density_loss_cotangent(cfg, uT, target):
    """loss = mean over interior cells of (rho_T - rho_target)^2 and its cotangent."""
    N = _abi.config_dim(cfg) + 2
    shape = grid_shape(cfg)
    mask = np.zeros(shape[:-1], dtype=bool)
    mask[(slice(2, -2),) * (len(shape) - 1)] = True
    r = (uT.reshape(shape)[..., 0] - target.reshape(shape)[..., 0])
    n = mask.sum()
    loss = float(np.sum(r[mask] ** 2) / n)
    lam = np.zeros(shape)
    lam[..., 0][mask] = 2 * r[mask] / n
    return loss, lam.reshape(-1)


@pytest.mark.parametrize("every", [1, 7, 30])
def test_checkpointed_gradient(hg, oracle_mod, every):
    cfg, u0 = kh_small()
    nsteps = 30
    s = hg.Solver(cfg)
    s.resetState(u0)
    cp = hg.Checkpoints(s, nsteps, every)
    cp.forward()
    dts = cp.dts()
    uT = s.getState().copy()
    # the checkpointed forward is the plain forward
    assert np.array_equal(uT, gpu_frozen(hg, cfg, u0, dts))
    target = uT + 1e-2 * np.random.default_rng(200).standard_normal(uT.size) * np.abs(uT)
    _, lamT = density_loss_cotangent(cfg, uT, target)
    dl = cuda(lamT)
    out = torch.empty_like(dl)
    torch.cuda.synchronize()
    cp.backward(dl.data_ptr(), out.data_ptr())
    s.synchronize()
    g = out.cpu().numpy()
    # against a chain of single-step products (same kernels: same bits)
    states = [u0]
    for dt in dts[:-1]:
        states.append(gpu_frozen(hg, cfg, states[-1], [dt]))
    lam = lamT
    for k in range(nsteps - 1, -1, -1):
        lam = gpu_vjp(hg, cfg, states[k], lam, dts[k])
    assert np.array_equal(g, lam)
    # against the torch restatement's gradient through the same 30 frozen steps
    g_ref, _ = torch_vjp(oracle_mod, cfg, u0, lamT, dts)
    assert rel(g, g_ref) <= 1e-9, rel(g, g_ref)
    cp.close()
    s.close()


def run_trajectory(hg, cfg, u0, nsteps, every=None, taped=False, dts=None):
    """final state, dts and lambda_0 of a density loss through nsteps steps"""
    s = hg.Solver(cfg)
    try:
        s.resetState(u0)
        cp = hg.Checkpoints(s, nsteps, every, taped=taped)
        cp.forward(dts)
        d = cp.dts()
        uT = s.getState().copy()
        target = uT + 1e-2 * np.random.default_rng(201).standard_normal(uT.size) * np.abs(uT)
        _, lamT = density_loss_cotangent(cfg, uT, target)
        dl = cuda(lamT)
        out = torch.empty_like(dl)
        torch.cuda.synchronize()
        cp.backward(dl.data_ptr(), out.data_ptr())
        s.synchronize()
        g = out.cpu().numpy()
        cp.close()
        return uT, d, g
    finally:
        s.close()


@pytest.mark.parametrize("integrator,frozen", [("RungeKutta2", False), ("RungeKutta4", False), ("ForwardEuler", False),
                                               ("RungeKutta3TVD", False), ("RungeKutta2Heun", True)])
def test_taped_trajectory_equals_checkpointed(hg, integrator, frozen):
    """The taped forward (every step's tape recorded as it runs, CFL dt taken on the
    device) gives the checkpointed forward's states, dts and gradient bit for bit, and
    its final state is the plain solver's."""
    cfg, u0 = kh_small(n=20, seed=103)
    cfg.integrator = _abi.INTEGRATORS.index(integrator)
    nsteps = 12
    dts = None
    if frozen:
        dts = np.array(run_trajectory(hg, cfg, u0, nsteps, every=5)[1]) * .9
    uA, dA, gA = run_trajectory(hg, cfg, u0, nsteps, every=5, dts=dts)
    uB, dB, gB = run_trajectory(hg, cfg, u0, nsteps, taped=True, dts=dts)
    assert np.array_equal(dA, dB)
    assert np.array_equal(uA, uB)
    assert np.array_equal(gA, gB)
    if not frozen:
        s = hg.Solver(cfg)
        s.resetState(u0)
        s.update(nsteps)
        assert np.array_equal(s.getState(), uB)
        s.close()


def test_taped_refuses_what_does_not_fit(hg):
    cfg, u0 = kh_small(n=508)
    s = hg.Solver(cfg)
    try:
        s.resetState(u0)
        with pytest.raises(hg.HgpuError):
            hg.Checkpoints(s, 1 << 20, taped=True)      # a million tapes of a 512^2 grid
    finally:
        s.close()


def drifting_flow(n=32, limiter="VanAlbada1"):
    """Smooth periodic flow whose velocities stay away from zero (u ~ .4, v ~ .3):
    no face changes its upwind side and VanAlbada1 has no kinks, so the rollout is
    differentiable and central differences converge to the adjoint."""
    size = (n + 4, n + 4)
    f = [ic.smooth_perturbation(size, seed=400 + k, amp=1.)[0] for k in range(4)]
    st = ic.build_state_euler(2, 1.4, 1. + .2 * f[0], .4 + .05 * f[1], .3 + .05 * f[2], 0., 1. + .1 * f[3])
    return _abi.make_config(solver="EulerRoe", size=size, boundary="PERIODIC", limiter=limiter,
                            integrator="RungeKutta2"), st.reshape(-1)


def test_checkpointed_gradient_vs_finite_differences(hg):
    """40 steps of a smooth drifting flow.  (On the Kelvin-Helmholtz state the normal
    velocity of many faces is within the noise of zero, so perturbations switch their
    upwind side -- a kink -- and the difference quotient is not a derivative.)"""
    cfg, u0 = drifting_flow()
    nsteps = 40
    s = hg.Solver(cfg)
    s.resetState(u0)
    cp = hg.Checkpoints(s, nsteps, 10)
    cp.forward()
    dts = cp.dts()
    uT = s.getState().copy()
    # target: the forward from u0 plus a smooth density perturbation of amplitude 1e-2
    target = uT.reshape(grid_shape(cfg)).copy()
    target[..., 0] += ic.smooth_perturbation((cfg.size[0], cfg.size[1]), seed=200)[0]
    target = target.reshape(-1)
    loss, lamT = density_loss_cotangent(cfg, uT, target)
    dl = cuda(lamT)
    out = torch.empty_like(dl)
    torch.cuda.synchronize()
    cp.backward(dl.data_ptr(), out.data_ptr())
    s.synchronize()
    g = out.cpu().numpy()
    rng = np.random.default_rng(300)
    for _ in range(4):
        d = rng.standard_normal(u0.size)
        d /= np.linalg.norm(d)
        lp, _ = density_loss_cotangent(cfg, gpu_frozen(hg, cfg, u0 + FD_EPS * d, dts), target)
        lm, _ = density_loss_cotangent(cfg, gpu_frozen(hg, cfg, u0 - FD_EPS * d, dts), target)
        fd = (lp - lm) / (2 * FD_EPS)
        ad = float(np.dot(g, d))
        assert abs(fd - ad) <= FD_TOL * abs(ad), (fd, ad)
    f_ms, b_ms = cp.times()
    assert f_ms > 0 and b_ms > 0
    cp.close()
    s.close()


def test_autograd_function(hg):
    from hydrodynamicsgpu_gb300.autograd import rollout
    cfg, u0 = kh_small(n=20, seed=102)
    s = hg.Solver(cfg)
    x = cuda(u0).requires_grad_(True)
    y = rollout(x, s, 12, every=5)
    w = cuda(np.random.default_rng(9).standard_normal(u0.size))
    (y * w).sum().backward()
    g = x.grad.cpu().numpy()
    # reference: checkpoint backward run directly
    s2 = hg.Solver(cfg)
    s2.resetState(u0)
    cp = hg.Checkpoints(s2, 12, 12)
    cp.forward()
    out = torch.empty_like(w)
    torch.cuda.synchronize()
    cp.backward(w.data_ptr(), out.data_ptr())
    s2.synchronize()
    assert np.array_equal(g, out.cpu().numpy())
    assert np.array_equal(y.detach().cpu().numpy(), s2.getState())
    cp.close()
    s.close()
    s2.close()


def test_adjoint_rejects_other_solvers(hg):
    cfg = _abi.make_config(solver="EulerHLLC", size=(20, 18))
    s = hg.Solver(cfg)
    with pytest.raises(hg.HgpuError):
        s.update_frozen_dt([1e-3])
    s.close()


def test_adjoint_rejects_fixed_dt(hg):
    """With useFixedDT an EulerRoe step keeps the eigenbasis the last CFL step left
    (Solver::update skips calcTimestep): the adjoint refuses such a solver."""
    cfg, u0 = kh_small()
    cfg.use_fixed_dt = 1
    cfg.fixed_dt = .001
    s = hg.Solver(cfg)
    try:
        s.resetState(u0)
        with pytest.raises(hg.HgpuError):
            hg.Checkpoints(s, 4, 2)
        with pytest.raises(hg.HgpuError):
            hg.Checkpoints(s, 4, taped=True)
        with pytest.raises(hg.HgpuError):
            s.update_frozen_dt([1e-3])
    finally:
        s.close()
