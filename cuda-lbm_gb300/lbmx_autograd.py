"""torch.autograd wrapper over the adjoint C-ABI (lbmx.Adjoint).

    J = lbmx_autograd.objective(gamma, omega, force, adj, nsteps)
    J.backward()        # gamma.grad, omega.grad, force.grad

gamma: float32 tensor [ny, nx] (the Brinkman field), omega: 0-d tensor,
force: tensor [2].  The forward runs the adjoint's own forward model (the
engine's step, checkpointed) and returns J as a float64 0-d tensor; the
backward runs the discrete adjoint.  No PyTorch autodiff touches the LBM:
the graph has this one node.
"""
import torch


class AdjointObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, gamma, omega, force, adj, nsteps):
        g = gamma.detach().to(torch.float32).contiguous()
        adj.set_gamma(g)
        adj.set_scalars(float(omega), float(force[0]), float(force[1]))
        J = adj.forward(int(nsteps))
        ctx.adj = adj
        ctx.gamma_meta = (gamma.shape, gamma.dtype, gamma.device)
        ctx.omega_meta = (omega.dtype, omega.device) if torch.is_tensor(omega) else None
        ctx.force_meta = (force.dtype, force.device) if torch.is_tensor(force) else None
        return torch.tensor(J, dtype=torch.float64, device=gamma.device)

    @staticmethod
    def backward(ctx, grad_out):
        shape, dtype, device = ctx.gamma_meta
        gg = torch.empty(shape, dtype=torch.float32, device=device)
        if device.type == "cuda":
            _, (gw, gfx, gfy) = ctx.adj.backward(gg)
        else:
            host, (gw, gfx, gfy) = ctx.adj.backward()
            gg = torch.from_numpy(host).reshape(shape)
        scale = grad_out.to(torch.float64)
        g_gamma = (gg.to(torch.float64) * scale.to(device)).to(dtype)
        g_omega = g_force = None
        if ctx.omega_meta is not None:
            g_omega = (scale * gw).to(ctx.omega_meta[0]).to(ctx.omega_meta[1])
        if ctx.force_meta is not None:
            g_force = (scale * torch.tensor([gfx, gfy], dtype=torch.float64, device=scale.device)).to(
                ctx.force_meta[0]).to(ctx.force_meta[1])
        return g_gamma, g_omega, g_force, None, None


def objective(gamma, omega, force, adj, nsteps):
    return AdjointObjective.apply(gamma, omega, force, adj, nsteps)
