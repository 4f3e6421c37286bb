"""A labelled initial condition beside the reference's PAO/KM3 generator.

``k4_unit_energy`` builds the literal spectrum of the precision-form
configuration: shell energy E(k) ∝ k^4 exp(-2 (k/K0)^2), uniform random phases
from a seeded NumPy generator, normalised so that the reference's energy
measure sum_m (|u1|^2 + |u3|^2) (the printed "Energy", turbo_simulator.py:
432-466, with weight 1 for kx = 0 and 2 otherwise) equals 1.  It is not the
reference generator (whose PAO shells follow k exp(-(k/K0)^2) and are not
normalised to exactly 1); results from it are labelled as such.
"""
from __future__ import annotations

import numpy as np


def k4_unit_energy(N: int, K0: float, seed: int):
    """Returns (om2 (N, N/2), uc_low (2, N, N/2)) complex64 in the reference layouts."""
    if N % 4 or N < 8:
        raise ValueError("N must be a multiple of 4 and >= 8")
    nh = N // 2
    kx = np.arange(nh, dtype=np.float64)[None, :]
    z = np.arange(N)
    kz = np.where(z < nh, z, z - N).astype(np.float64)[:, None]
    k2 = kx * kx + kz * kz
    k = np.sqrt(k2)
    rng = np.random.default_rng(seed)
    phase = np.exp(2j * np.pi * rng.random((N, nh)))
    # |om|^2 per mode so that each shell carries E(k) spread over its ~2 pi k modes
    with np.errstate(divide="ignore", invalid="ignore"):
        e_k = k ** 4 * np.exp(-2.0 * (k / K0) ** 2)
        om_amp2 = np.where(k2 > 0, e_k * k2 / (2.0 * np.pi * np.maximum(k, 1e-300)), 0.0)
    keep = (k2 > 0) & (k <= nh) & (z[:, None] != nh)
    om = np.where(keep, np.sqrt(om_amp2) * phase, 0.0)
    # Hermitian kx = 0 column: om(0, -kz) = conj(om(0, kz))
    for zz in range(1, nh):
        om[N - zz, 0] = np.conj(om[zz, 0])
    # velocity from the inversion used by the step (turbo_simulator.py:1555-1585)
    u = np.zeros_like(om)
    v = np.zeros_like(om)
    inv = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    u[:, 1:] = -1j * kz * om[:, 1:] * inv[:, 1:]
    v[:, 1:] = 1j * kx[:, 1:] * om[:, 1:] * inv[:, 1:]
    kz0 = kz[:, 0]
    u[:, 0] = np.where(kz0 != 0, -1j * om[:, 0] / np.where(kz0 != 0, kz0, 1.0), 0.0)
    w = np.where(kx == 0, 1.0, 2.0)
    energy = float((w * (np.abs(u) ** 2 + np.abs(v) ** 2)).sum())
    scale = 1.0 / np.sqrt(energy)
    om2 = (om * scale).astype(np.complex64)
    uc = np.stack([u * scale, v * scale]).astype(np.complex64)
    return om2, uc
