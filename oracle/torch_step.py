"""Plain torch.fft re-implementation of the LS-IMEX-RK3 step -- TEST INFRASTRUCTURE.

Used only by tests/ as the reference gradient for the hand-written adjoint:
autograd differentiates this restatement of turbo_simulator.py's step
(pad / irfft2(norm='forward') / products / rfft2 / gather / IMEX update,
TS:1378-1943) and of the final-palinstrophy loss 1/2 sum w' K2 |om|^2.
"""
from __future__ import annotations

import torch

ALPHA = (8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0)
BETA = (0.0, -17.0 / 60.0, -5.0 / 12.0)


class Grid:
    def __init__(self, N, dtype=torch.float64):
        self.N, self.Nh, self.M = N, N // 2, 3 * N // 2
        self.rdt = dtype
        kx = torch.arange(self.Nh, dtype=dtype)[None, :]
        z = torch.arange(N)
        kz = torch.where(z < self.Nh, z, z - N).to(dtype)[:, None]
        self.kx, self.kz = kx, kz
        self.K2 = kx * kx + kz * kz
        self.GA = kz * kx
        self.G2 = kz * kz - kx * kx
        self.divxz = 1.0 / float(self.M * self.M)
        k2s = torch.where(self.K2 > 0, self.K2, torch.ones_like(self.K2))
        self.cu = torch.where(kx > 0, -1j * kz / k2s, torch.zeros((), dtype=torch.complex128))
        kz0 = torch.where(kz != 0, kz, torch.ones_like(kz))
        cu0 = torch.where((kz != 0), -1j / kz0, torch.zeros((), dtype=torch.complex128))
        self.cu = torch.where(kx == 0, cu0.expand_as(self.cu), self.cu)
        self.cv = torch.where(kx > 0, 1j * kx / k2s, torch.zeros((), dtype=torch.complex128))
        self.rows = torch.cat([torch.arange(self.Nh), torch.arange(N, N + self.Nh)])
        self.w = torch.where(kx == 0, 1.0, 2.0).to(dtype)

    def pad(self, band):
        X = torch.zeros((self.M, self.M // 2 + 1), dtype=band.dtype)
        return X.index_put((self.rows[:, None], torch.arange(self.Nh)[None, :]), band)

    def phys(self, band):
        return torch.fft.irfft2(self.pad(band), s=(self.M, self.M), norm="forward")

    def gather(self, spec):
        return spec[self.rows][:, : self.Nh]


def rk3_step(g: Grid, om, f, dt, visc):
    for a, b in zip(ALPHA, BETA):
        u = g.phys(g.cu * om)
        v = g.phys(g.cv * om)
        A = g.gather(torch.fft.rfft2(u * u - v * v))
        B = g.gather(torch.fft.rfft2(u * v))
        fn = g.divxz * (g.GA * A + g.G2 * B)
        fn = torch.cat([fn[: g.Nh], torch.zeros_like(fn[g.Nh:g.Nh + 1]), fn[g.Nh + 1:]])
        om = ((1.0 - g.K2 * (b * dt * visc)) * om + (a * dt) * fn + (b * dt) * f) / (1.0 + g.K2 * (a * dt * visc))
        f = fn
    return om, f


def palinstrophy(g: Grid, om):
    return 0.5 * (g.w * g.K2 * (om.real ** 2 + om.imag ** 2)).sum()


def loss_and_grad(om0, N, dt, visc, nsteps):
    """Final palinstrophy after nsteps fixed-dt RK3 steps and its autograd gradient."""
    g = Grid(N)
    om = torch.as_tensor(om0, dtype=torch.complex128).clone().requires_grad_(True)
    x, f = om, torch.zeros_like(om)
    for _ in range(nsteps):
        x, f = rk3_step(g, x, f, dt, visc)
    L = palinstrophy(g, x)
    L.backward()
    return float(L.detach()), om.grad.numpy()
