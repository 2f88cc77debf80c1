"""torch.autograd.Function over the EulerRoe rollout (FP64) through the C ABI.

Thin ctypes wrapper used for gradient checks: forward runs `nsteps` steps of a
Solver from u0 with checkpoints every `every` steps (the dt of each step is the
CFL value, or the given frozen values) and returns u_T; backward maps dL/du_T to
dL/du0 with hgpu_checkpoint_backward.  dt is held at the forward's values (it is
not differentiated).  Tensors are full FP64 states (ghosts included) on the
solver's CUDA device."""
import numpy as np
import torch

from . import Checkpoints


class RoeRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, solver, nsteps, every, dts):
        if u0.dtype != torch.float64 or not u0.is_cuda:
            raise TypeError("u0 must be a CUDA float64 tensor")
        solver.resetState(u0.detach().cpu().numpy())
        cp = Checkpoints(solver, nsteps, every)
        cp.forward(None if dts is None else np.asarray(dts, dtype=np.float64))
        ctx.cp = cp
        ctx.dts = cp.dts()
        uT = torch.from_numpy(solver.getState().copy()).to(u0.device)
        return uT

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous().to(torch.float64)
        out = torch.empty_like(g)
        torch.cuda.synchronize(g.device)
        ctx.cp.backward(g.data_ptr(), out.data_ptr())
        ctx.cp.solver.synchronize()
        return out, None, None, None, None


def rollout(u0, solver, nsteps, every=20, dts=None):
    """u_T as a differentiable function of u0 (see RoeRollout)."""
    return RoeRollout.apply(u0, solver, nsteps, every, dts)
