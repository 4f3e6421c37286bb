"""torch.autograd.Function over the hand-written adjoint of the DNS step.

    L = PalinstrophyLoss.apply(om0, N, precision, dt, visc, nsteps, ckpt_every)

om0 is the initial spectral vorticity (N, N/2) as a complex torch tensor; a
CUDA tensor is read by the library in place (no host round trip), a CPU tensor
is uploaded.  L = 1/2 sum w' K2 |om|^2 of the field after nsteps fixed-dt
LS-IMEX-RK3 steps.  When om0 needs no gradient, forward only steps the field
and evaluates L.  When it does, forward makes one pal_adjoint_palinstrophy call,
which returns L and dL/d om0 together (its own checkpointed forward sweep plus
the reversed stages), and backward scales that gradient by grad_output
(convention dL = Re sum conj(g) d om0, PyTorch's for complex inputs).
"""
from __future__ import annotations

import numpy as np
import torch

from .turbo_simulator import Field


def _final_palinstrophy(om: np.ndarray, N: int) -> float:
    om = om.astype(np.complex128)
    kx = np.arange(N // 2)[None, :]
    kz = np.fft.fftfreq(N, 1.0 / N)[:, None]
    w = np.where(kx == 0, 1.0, 2.0)
    return 0.5 * float((w * (kx * kx + kz * kz) * np.abs(om) ** 2).sum())


class PalinstrophyLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, om0, N, precision="fp32", dt=2e-3, visc=2e-4, nsteps=200, ckpt_every=20):
        N = int(N)
        F = Field(N, precision, 1.0 / visc, 0.5)
        try:
            cdt = torch.complex64 if precision == "fp32" else torch.complex128
            src = om0.detach()
            if src.is_cuda:
                src = src.to(cdt).contiguous()
                torch.cuda.current_stream(src.device).synchronize()
                F.set_state_device(src.data_ptr())
            else:
                F.set_state(src.numpy(), None, None)
            F.set_scalar("visc", float(visc))
            F.set_scalar("dt", float(dt))
            if ctx.needs_input_grad[0]:
                loss, grad = F.adjoint_palinstrophy(int(nsteps), int(ckpt_every))
                ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(grad)).to(om0.device))
            else:
                F.step("LS_IMEX_RK3", int(nsteps), update=0)
                loss = _final_palinstrophy(F.om2(), N)
        finally:
            F.close()
        return torch.tensor(loss, dtype=torch.float64, device=om0.device)

    @staticmethod
    def backward(ctx, grad_output):
        (g,) = ctx.saved_tensors
        return (grad_output * g).to(g.dtype), None, None, None, None, None, None
