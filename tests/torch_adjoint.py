"""Test-only torch.autograd.Function over the library's differentiable trajectory.

Not part of the product: the C ABI (bh_adjoint_forward / bh_step_backward) is the interface;
this wrapper only lets a test write the loss in torch and check that loss.backward() hands the
library's gradients back through autograd. Tensors are host (CPU) float32; the library copies
them to the GPU itself.
"""
import numpy as np
import torch


class Trajectory(torch.autograd.Function):
    """(x0 (n,3), v0 (n,3), m (n,)) -> (x_N, v_N) after nsteps KDK steps of the tree force."""

    @staticmethod
    def forward(ctx, x0, v0, m, sim, params, nsteps, every):
        n = x0.shape[0]
        pm = np.zeros((n, 4), np.float32)
        pm[:, :3] = x0.detach().cpu().numpy()
        pm[:, 3] = m.detach().cpu().numpy()
        v4 = np.zeros((n, 4), np.float32)
        v4[:, :3] = v0.detach().cpu().numpy()
        sim.set_bodies(pm, v4)
        sim.adjoint_forward(params, nsteps, every)
        p, v, _ = sim.get_bodies()
        ctx.sim = sim
        return torch.from_numpy(p[:, :3].copy()), torch.from_numpy(v[:, :3].copy())

    @staticmethod
    def backward(ctx, gx, gv):
        gxn = None if gx is None else gx.detach().cpu().numpy()
        gvn = None if gv is None else gv.detach().cpu().numpy()
        gx0, gv0, gm = ctx.sim.step_backward(gxn, gvn)
        return (torch.from_numpy(gx0[:, :3].copy()), torch.from_numpy(gv0[:, :3].copy()), torch.from_numpy(gm),
                None, None, None, None)


def trajectory(x0, v0, m, sim, params, nsteps, every):
    return Trajectory.apply(x0, v0, m, sim, params, nsteps, every)
