"""torch.autograd.Function over the library's hand-written adjoint.

    from lbmcl_gb300.adjoint import cavity_loss
    lid = torch.full((dim, dim), 0.05, dtype=torch.float64, requires_grad=True)
    tau = torch.tensor(0.53, dtype=torch.float64, requires_grad=True)
    J = cavity_loss(lid, tau, None, dim=64, iterations=2000, checkpoint_every=100,
                    plane_y=32, target=target_ux)
    J.backward()        # lid.grad, tau.grad

The forward pass runs the D3Q19 cavity on the GPU through the C ABI
(lbm_adjoint_forward, with checkpoints) and returns the mid-plane loss
J = mean over the FLUID sites of plane y of (u_x - target)^2; the backward
pass runs lbm_adjoint_backward (hand-written adjoint kernels, checkpoint
segments recomputed).  Controls: the per-column lid velocity `lid` [y, x],
the relaxation time `tau`, and optionally the initial populations `f0` (the
LBM_DUMP_F layout, i.e. what Lattice.f() returns; None = the equilibrium
initial state, which then depends on the lid).  All tensors live on the
host; the library copies them.
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi


class _CavityLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, lid, tau, f0, opts):
        dim = opts["dim"]
        # the forward records the last segments' linearisation points for a
        # backward sweep without a tau gradient; with one it would not use them
        L = capi.Lattice(dim, velocity=0.0, precision=opts.get("precision", "fp32"),
                         stride=opts.get("stride"), lid=lid.detach().cpu().numpy().reshape(-1),
                         tau=float(tau), seed=opts.get("seed", 0), noise_sigma=opts.get("noise", 0.0),
                         device=opts.get("device", 0),
                         adjoint_tail_segments=-1 if ctx.needs_input_grad[1] else 0)
        if f0 is not None:
            L.load_f(f0.detach().cpu().numpy())
        L.adjoint_set_loss(opts["plane_y"], opts.get("target"))
        loss = L.adjoint_forward(opts["iterations"], opts.get("checkpoint_every", 1))
        ctx.lattice = L
        ctx.has_f0 = f0 is not None
        ctx.dtypes = (lid.dtype, tau.dtype, f0.dtype if f0 is not None else None)
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        L = ctx.lattice
        # without a tau gradient the sweep stores only velocities / lid
        # densities per iteration instead of full states
        want_tau = bool(ctx.needs_input_grad[1])
        g_tau, g_lid, g_f0 = L.adjoint_backward(float(grad_out), want_f0=ctx.has_f0, want_tau=want_tau)
        L.close()
        ctx.lattice = None
        lt, tt, ft = ctx.dtypes
        out_f0 = torch.from_numpy(np.ascontiguousarray(g_f0)).to(ft) if ctx.has_f0 else None
        out_tau = torch.tensor(g_tau, dtype=tt) if want_tau else None
        return (torch.from_numpy(g_lid).to(lt), out_tau, out_f0, None)


def cavity_loss(lid: torch.Tensor, tau: torch.Tensor, f0, *, dim: int, iterations: int, plane_y: int,
                target=None, checkpoint_every: int = 1, precision: str = "fp32", stride=None, seed: int = 0,
                noise: float = 0.0, device: int = 0) -> torch.Tensor:
    """Mid-plane velocity loss of a `dim`^3 cavity after `iterations` steps
    (differentiable in lid, tau and f0)."""
    opts = dict(dim=dim, iterations=iterations, plane_y=plane_y, target=target, checkpoint_every=checkpoint_every,
                precision=precision, stride=stride, seed=seed, noise=noise, device=device)
    return _CavityLoss.apply(lid, tau, f0, opts)
