"""torch.autograd binding of the adjoint: the MR advection time loop as a
differentiable function of the initial leaf values u0 and the velocity a.

    adj = samurai_gb300.Adjoint(u, checkpoint_every=16)
    uT = advection_loop(u0, a, adj, n_steps, eps, regularity, dt)
    J = (vol * (uT - target) ** 2).sum()
    J.backward()          # u0.grad, a.grad from the discrete adjoint

The forward records the loop with adaptation (its mesh sequence); the
gradient is that of the loop on the recorded meshes.  Tensors may live on any
device; values cross the C ABI through host arrays.
"""
import numpy as np
import torch


class AdvectionLoop(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, a, adj, n_steps, eps, regularity, dt, scheme):
        uT = adj.record(u0.detach().to("cpu", torch.float64).numpy(), n_steps, eps, regularity,
                        a.detach().to("cpu", torch.float64).numpy(), dt, scheme)
        ctx.adj = adj
        ctx.u0_meta = (u0.device, u0.dtype)
        ctx.a_meta = (a.device, a.dtype)
        return torch.from_numpy(uT).to(device=u0.device, dtype=u0.dtype)

    @staticmethod
    def backward(ctx, gT):
        g0, ga = ctx.adj.backward(np.ascontiguousarray(gT.detach().to("cpu", torch.float64).numpy()))
        (ud, ut), (ad, at) = ctx.u0_meta, ctx.a_meta
        return (torch.from_numpy(g0).to(device=ud, dtype=ut), torch.from_numpy(ga).to(device=ad, dtype=at),
                None, None, None, None, None, None)


def advection_loop(u0, a, adj, n_steps, eps, regularity, dt, scheme=0):
    """uT = the time loop of n_steps from u0 (leaf values of adj's initial mesh)"""
    return AdvectionLoop.apply(u0, a, adj, n_steps, eps, regularity, dt, scheme)
