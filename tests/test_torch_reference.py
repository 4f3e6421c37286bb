"""The torch.fft restatement used as the gradient reference agrees with the
NumPy oracle's forward step (CPU, FP64)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import dns_oracle as do  # noqa: E402
from oracle import pao_generator as pg  # noqa: E402
from oracle import torch_step as tsr  # noqa: E402


def test_torch_step_matches_oracle():
    g = pg.generate(32, 6.0, 1e4, 5, "KM3")
    dt, visc = 2e-3, 2e-4
    S = do.OracleState(32, g["om2"], None if False else np.zeros((2, 32, 16), np.complex64), visc, 0.5)
    S.dt = dt
    # velocity from the om2 inversion, as the adjoint's forward uses it
    do.reconstruct_velocity(S)
    do.step2a(S)
    for _ in range(3):
        do.rk3(S)
    G = tsr.Grid(32)
    om = torch.as_tensor(g["om2"], dtype=torch.complex128)
    f = torch.zeros_like(om)
    for _ in range(3):
        om, f = tsr.rk3_step(G, om, f, dt, visc)
    assert do.rel_l2(S.om2, om.numpy()) < 1e-13
