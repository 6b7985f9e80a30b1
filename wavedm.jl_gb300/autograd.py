"""torch.autograd.Function over the checkpointed adjoint (wdm_adjoint).

The Python analogue of the Julia ChainRulesCore.rrule in julia/WaveDMGB300.jl:
the forward returns L = sum(|psi_N|^2 - rho_target)^2 dV of an nsteps Strang run
from psi0, the backward returns dL/dpsi0 (as dL/dRe + i dL/dIm, torch's
convention for complex leaves) and dL/da for a tide a * tidal_dir.
"""
from __future__ import annotations

import numpy as np
import torch

from .core import SPEContext


class EvolveLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx_, psi0, amp, spe_ctx: SPEContext, nsteps, dt, rho_target, tidal_dir, ckpt_every=20):
        D = np.asarray(tidal_dir, np.float64)
        spe_ctx.set_psi(psi0.detach().contiguous())
        spe_ctx.set_tidal([float(amp) * D])
        if not (ctx_.needs_input_grad[0] or ctx_.needs_input_grad[1]):
            # no gradient wanted: the forward run alone (the adjoint costs ~2.5 of them)
            spe_ctx.step(nsteps, dt)
            rho = torch.empty(psi0.shape, dtype=torch.float32, device=psi0.device)
            spe_ctx.get_rho(rho)
            diff = rho.double() - torch.as_tensor(rho_target, device=psi0.device).double()
            loss = (diff * diff).sum() * spe_ctx.cell_volume
            spe_ctx.set_psi(psi0.detach().contiguous())  # psi is left at psi0, as wdm_adjoint leaves it
            return loss.to(torch.float64)
        grad = torch.empty_like(psi0)
        loss, _, damp = spe_ctx.adjoint(nsteps, dt, rho_target, ckpt_every=ckpt_every, tidal_dir=D, grad_out=grad)
        ctx_.save_for_backward(grad)
        ctx_.damp = float(damp)
        return torch.tensor(float(loss), dtype=torch.float64, device=psi0.device)

    @staticmethod
    def backward(ctx_, gout):
        (grad,) = ctx_.saved_tensors
        g = gout.to(torch.float32)
        return grad * g, (g.double() * ctx_.damp).to(torch.float64), None, None, None, None, None, None


def evolve_loss(psi0, amp, spe_ctx, nsteps, dt, rho_target, tidal_dir, ckpt_every=20):
    """L(psi0, amp) with autograd support through the library's adjoint."""
    return EvolveLoss.apply(psi0, amp, spe_ctx, nsteps, dt, rho_target, tidal_dir, ckpt_every)
