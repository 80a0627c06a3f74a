"""torch.autograd binding of the adjoint: the MR advection time loop as a
differentiable function of the initial leaf values u0 and the velocity a.

    adj = samurai_gb300.Adjoint(u, checkpoint_every=16)
    uT = advection_loop(u0, a, adj, n_steps, eps, regularity, dt)
    J = (vol * (uT - target) ** 2).sum()
    J.backward()          # u0.grad, a.grad from the discrete adjoint

The forward records the loop with adaptation (its mesh sequence); the
gradient is that of the loop on the recorded meshes.  FP64 tensors on the
mesh's GPU cross the C ABI as device pointers (no host round trip); tensors
elsewhere, or of another type, are staged through FP64 host buffers.
"""
import torch


def _on_device(t):
    return t.is_cuda and t.dtype == torch.float64


def _as_input(t):
    """t's values, contiguous FP64, where the library can read them"""
    t = t.detach()
    if _on_device(t):
        t = t.contiguous()
        # the library reads on its own stream: the producer's work must be done
        torch.cuda.current_stream(t.device).synchronize()
        return t
    return t.to("cpu", torch.float64).contiguous()


def _output_like(n, ref):
    if _on_device(ref):
        return torch.empty(n, dtype=torch.float64, device=ref.device)
    return torch.empty(n, dtype=torch.float64)


class AdvectionLoop(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, a, adj, n_steps, eps, regularity, dt, scheme):
        src = _as_input(u0)
        av = a.detach().to("cpu", torch.float64).numpy()
        nT = adj.record_ptr(src.data_ptr(), n_steps, eps, regularity, av, dt, scheme)
        uT = _output_like(nT, u0)
        adj.final_ptr(uT.data_ptr(), nT)
        ctx.adj = adj
        ctx.u0_meta = (u0.device, u0.dtype, _on_device(u0))
        ctx.a_meta = (a.device, a.dtype)
        return uT.to(device=u0.device, dtype=u0.dtype)

    @staticmethod
    def backward(ctx, gT):
        ud, ut, on_dev = ctx.u0_meta
        n0, _, _ = ctx.adj.counts()
        g_in = _as_input(gT)
        g0 = torch.empty(n0, dtype=torch.float64, device=ud) if on_dev else torch.empty(n0, dtype=torch.float64)
        ga = ctx.adj.backward_ptr(g_in.data_ptr(), g0.data_ptr())
        ad, at = ctx.a_meta
        return (g0.to(device=ud, dtype=ut), torch.from_numpy(ga).to(device=ad, dtype=at), None, None, None, None, None, None)


def advection_loop(u0, a, adj, n_steps, eps, regularity, dt, scheme=0):
    """uT = the time loop of n_steps from u0 (leaf values of adj's initial mesh)"""
    return AdvectionLoop.apply(u0, a, adj, n_steps, eps, regularity, dt, scheme)
