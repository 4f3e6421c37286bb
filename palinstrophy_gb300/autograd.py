"""torch.autograd.Function over the hand-written adjoint of the DNS step.

    L = PalinstrophyLoss.apply(om0, N, precision, dt, visc, nsteps, ckpt_every)

om0 is the initial spectral vorticity (N, N/2) as a complex torch tensor (any
device; it is copied to the host for the C ABI).  Forward runs nsteps fixed-dt
LS-IMEX-RK3 steps on the GPU and returns L = 1/2 sum w' K2 |om|^2 of the final
field; backward returns grad_output * dL/d om0 from pal_adjoint_palinstrophy
(gradient convention dL = Re sum conj(g) d om0, PyTorch's for complex inputs).
"""
from __future__ import annotations

import numpy as np
import torch

from .turbo_simulator import Field


class PalinstrophyLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, om0, N, precision="fp32", dt=2e-3, visc=2e-4, nsteps=200, ckpt_every=20):
        F = Field(int(N), precision, 1.0 / visc, 0.5)
        try:
            F.set_state(om0.detach().cpu().numpy(), None, None)
            F.set_scalar("visc", float(visc))
            F.set_scalar("dt", float(dt))
            loss, grad = F.adjoint_palinstrophy(int(nsteps), int(ckpt_every))
        finally:
            F.close()
        ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(grad)).to(om0.device))
        return torch.tensor(loss, dtype=torch.float64, device=om0.device)

    @staticmethod
    def backward(ctx, grad_output):
        (g,) = ctx.saved_tensors
        return (grad_output * g).to(torch.complex128 if g.dtype == torch.complex128 else g.dtype), \
            None, None, None, None, None, None
