"""The labelled k^4 exp(-2(k/K0)^2) unit-energy start (no GPU needed)."""
import numpy as np

from palinstrophy_gb300.initial import k4_unit_energy


def test_unit_energy_and_structure():
    N, K0 = 128, 15.0
    om2, uc = k4_unit_energy(N, K0, 4895)
    nh = N // 2
    w = np.where(np.arange(nh) == 0, 1.0, 2.0)[None, :]
    e = float((w * (np.abs(uc[0].astype(np.complex128)) ** 2 + np.abs(uc[1].astype(np.complex128)) ** 2)).sum())
    assert abs(e - 1.0) < 1e-6
    # Hermitian kx = 0 column, zero (0,0) and z = N/2 row
    for z in range(1, nh):
        assert om2[N - z, 0] == np.conj(om2[z, 0])
    assert om2[0, 0] == 0 and not om2[nh].any()
    # divergence free: kx u + kz v = 0
    kx = np.arange(nh)[None, :]
    kz = np.fft.fftfreq(N, 1.0 / N)[:, None]
    div = kx * uc[0].astype(np.complex128) + kz * uc[1].astype(np.complex128)
    assert np.abs(div).max() < 1e-5 * np.abs(uc).max() * N
    # shell energy peaks near K0
    k = np.sqrt(kx * kx + kz * kz)
    shells = np.bincount(np.rint(k).astype(int).ravel(),
                         weights=(w * (np.abs(uc[0]) ** 2 + np.abs(uc[1]) ** 2)).ravel())
    assert abs(int(np.argmax(shells)) - K0) <= 2


def test_seeded_and_reproducible():
    a = k4_unit_energy(64, 10.0, 7)
    b = k4_unit_energy(64, 10.0, 7)
    c = k4_unit_energy(64, 10.0, 8)
    assert np.array_equal(a[0], b[0]) and not np.array_equal(a[0], c[0])
