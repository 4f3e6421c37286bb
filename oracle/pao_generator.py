"""Oracle restatement of palinstrophy's PAO / KM3 initial-condition generator.

TEST INFRASTRUCTURE ONLY.  Nothing in ``palinstrophy_gb300`` imports this
module; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may use it, to check the product's own generator against it.

It follows the reference generator step by step so that, on the same machine,
it reproduces the reference arrays:

* seeded Fortran LCG (IMM=420029, IT=2017, ID=5011), 97 warm-up draws and a
  97-entry shuffle table            -- turbo_simulator.py:241-261
* random-phase PAO velocity modes, |u|^2 ~ exp(-(k/K0)^2)/(pi K0^2) with the
  divergence-free split u = -(gamma/alfa) w       -- turbo_simulator.py:274-318
* zero (0,0) mode, Hermitian fill of the kx=0 column, zero row z=N/2
                                                  -- turbo_simulator.py:320-334
* KM3 shell rescale with the sin-hash jitter      -- turbo_simulator.py:195-204,
                                                     336-427
* visc = float32(1/Re), moment sums A1..A7        -- turbo_simulator.py:432-470
* om2 = i (gamma*u - alfa*w)  (dnsCudaCalcom)     -- turbo_simulator.py:1314-1361

The float32 arithmetic of the reference (NumPy float32 scalars) is kept in
float32 here, the shell sums in float64 in the reference's serial order.
"""
from __future__ import annotations

import math

import numpy as np

LCG_IMM = 420029
LCG_IT = 2017
LCG_ID = 5011
PI32 = np.float32(3.14159265358979)


def hash01(x: int, z: int, seed: int, salt: int) -> float:
    """Sin-hash in [0,1) used for KM3 jitter and phases (turbo_simulator.py:195-204)."""
    a = (float(x) + 1.0) * 12.9898 + (float(z) + 1.0) * 78.233
    a = a + (float(seed) + 1.0) * 0.010001
    a = a + (float(salt) + 1.0) * 37.719
    s = math.sin(a) * 43758.5453123
    return s - math.floor(s)


def wavenumbers(N: int):
    """alfa (kx = 0..N/2-1) and gamma (kz in FFT order, gamma[N/2] = -N/2)."""
    nh = N // 2
    alfa = np.arange(nh, dtype=np.float32)
    gamma = np.zeros(N, dtype=np.float32)
    for z in range(1, nh + 1):
        gamma[z] = np.float32(z)
        gamma[N - z] = -gamma[z]
    return alfa, gamma


def _random_modes(N, K0, seed, alfa, gamma, km3):
    """PAO random spectrum; returns (UR[x, z, comp] complex64, seed_out)."""
    nh = N // 2
    s = int(seed)
    for _ in range(97):
        s = (s * LCG_IMM + LCG_IT) % LCG_ID
    table = np.zeros(97, dtype=np.float32)
    for i in range(97):
        s = (s * LCG_IMM + LCG_IT) % LCG_ID
        table[i] = np.float32(s) / np.float32(LCG_ID)

    norm = PI32 * K0 * K0
    floor2 = np.float32(1.0e-40)
    ur = np.zeros((nh, N, 2), dtype=np.complex64)
    for z in range(N):
        gz = gamma[z]
        for x in range(nh):
            s = (s * LCG_IMM + LCG_IT) % LCG_ID
            r = np.float32(s) / np.float32(LCG_ID)
            idx = min(max(int(float(r) * 97.0), 0), 96)
            v = table[idx]
            table[idx] = r
            th = np.float32(2.0) * PI32 * v
            phase = np.complex64(np.cos(th) + 1j * np.sin(th))
            ax = alfa[x]
            k2 = np.float32(ax * ax + gz * gz)
            k = np.float32(np.sqrt(k2)) if k2 > 0.0 else np.float32(0.0)
            ratio = (k / K0) * (k / K0)
            if ax == 0.0:
                e2 = np.float32(np.exp(-ratio) / norm)
                if km3 and e2 < floor2:
                    e2 = floor2
                ur[x, z, 1] = 0
                ur[x, z, 0] = np.complex64(np.float32(np.sqrt(e2))) * phase
            else:
                den = np.float32(1.0) + (gz * gz) / (ax * ax)
                e2 = np.float32(np.exp(-ratio) / (den * norm))
                if km3 and e2 < floor2:
                    e2 = floor2
                w = np.complex64(np.float32(np.sqrt(e2))) * phase
                ur[x, z, 1] = w
                ur[x, z, 0] = np.complex64(-(gz / ax)) * w
    ur[0, 0, :] = 0
    for z in range(1, nh):
        ur[0, N - z, :] = np.conj(ur[0, z, :])
    ur[:, nh, :] = 0
    return ur, s


def _km3_rescale(ur, N, K0, seed_init, alfa, gamma):
    """Shell-rescale toward E(k) ~ k^-3 keeping the PAO total energy."""
    nh = N // 2
    knyq = float(nh)
    e_shell = np.zeros(nh + 1, dtype=np.float64)
    w_shell = np.zeros(nh + 1, dtype=np.float64)
    for x in range(nh):
        m = 1.0 if x == 0 else 2.0
        ax2 = float(alfa[x]) * float(alfa[x])
        for z in range(N):
            u1, u3 = ur[x, z, 0], ur[x, z, 1]
            p1 = float(u1.real) * float(u1.real) + float(u1.imag) * float(u1.imag)
            p3 = float(u3.real) * float(u3.real) + float(u3.imag) * float(u3.imag)
            k = math.sqrt(ax2 + float(gamma[z]) * float(gamma[z]))
            sh = int(k + 0.5)
            if 0.0 < k <= knyq and sh <= nh:
                e_shell[sh] += m * (p1 + p3)
                zh = N - z if (x == 0 and z > nh) else z
                w_shell[sh] += m * (0.75 + 0.50 * hash01(x, zh, seed_init, 17))
    k0 = max(float(K0), 1.0)
    target = np.zeros(nh + 1, dtype=np.float64)
    for sh in range(1, nh + 1):
        k = float(sh)
        if k < k0:
            lo = k / k0
            target[sh] = (lo * lo * lo * lo) / (k0 * k0 * k0)
        else:
            target[sh] = 1.0 / (k * k * k)
    e_orig = 0.0
    e_target = 0.0
    for sh in range(1, nh + 1):
        e_orig += e_shell[sh]
        e_target += target[sh]
    if not (e_orig > 0.0 and e_target > 0.0):
        return
    scale = e_orig / e_target
    for x in range(nh):
        ax = float(alfa[x])
        ax2 = ax * ax
        for z in range(N):
            gz = float(gamma[z])
            gz2 = gz * gz
            k = math.sqrt(ax2 + gz2)
            sh = int(k + 0.5)
            if 0.0 < k <= knyq and sh <= nh and w_shell[sh] > 0.0:
                zh, sign = z, 1.0
                if x == 0 and z > nh:
                    zh, sign = N - z, -1.0
                jit = 0.75 + 0.50 * hash01(x, zh, seed_init, 17)
                e_mode = (scale * target[sh]) * jit / w_shell[sh]
                th = sign * 2.0 * math.pi * hash01(x, zh, seed_init, 53)
                ph = np.complex64(math.cos(th) + 1j * math.sin(th))
                if ax == 0.0:
                    ur[x, z, 0] = np.complex64(math.sqrt(e_mode)) * ph
                    ur[x, z, 1] = 0
                else:
                    w = np.complex64(math.sqrt(e_mode / (1.0 + gz2 / ax2))) * ph
                    ur[x, z, 0] = np.complex64(-gz / ax) * w
                    ur[x, z, 1] = w
            else:
                ur[x, z, :] = 0


def _moments(ur, alfa, gamma):
    """Q2 (energy), W2 (enstrophy-like WiWi) and E110 as the reference sums them."""
    nh, N = ur.shape[0], ur.shape[1]
    a1 = a2 = a3 = a4 = a5 = a6 = a7 = 0.0
    for x in range(nh):
        ax2 = float(alfa[x]) * float(alfa[x])
        m = 1.0 if x == 0 else 2.0
        for z in range(N):
            u1, u3 = ur[x, z, 0], ur[x, z, 1]
            p1 = float(u1.real) * float(u1.real) + float(u1.imag) * float(u1.imag)
            p3 = float(u3.real) * float(u3.real) + float(u3.imag) * float(u3.imag)
            gz2 = float(gamma[z]) * float(gamma[z])
            k2 = ax2 + gz2
            a1 += m * p1
            a2 += m * p3
            a3 += m * p1 * ax2
            a4 += m * p1 * gz2
            a5 += m * p3 * ax2
            a6 += m * p3 * gz2
            a7 += m * (p1 + p3) * k2 * k2
    return {"Q2": a1 + a2, "W2": a3 + a4 + a5 + a6, "A1": a1, "A7": a7}


def generate(N: int, K0: float, Re: float, seed: int, spectrum: str = "KM3"):
    """Initial spectral state exactly as create_dns_state builds it.

    Returns a dict with
      om2      (N, N/2) complex64  -- spectral vorticity, [z, kx]
      uc_low   (2, N, N/2) complex64 -- velocity modes u1, u3 in uc_full's low band
      visc     float32(1/Re)
      seed_out, Q2 (printed 'Energy'), W2 (printed 'WiWi')
    """
    if N % 4 or N < 8:
        raise ValueError("N must be a multiple of 4 and >= 8")
    spectrum = spectrum.upper()
    if spectrum not in ("KM3", "PAO"):
        raise ValueError(f"unknown start spectrum {spectrum!r}")
    km3 = spectrum == "KM3"
    alfa, gamma = wavenumbers(N)
    k0 = np.float32(K0)
    ur, seed_out = _random_modes(N, k0, int(seed), alfa, gamma, km3)
    if km3:
        _km3_rescale(ur, N, k0, int(seed), alfa, gamma)
    mom = _moments(ur, alfa, gamma)
    uc_low = np.ascontiguousarray(np.transpose(ur, (2, 1, 0)))  # (2, N, N/2)
    ax = alfa[None, :]
    gz = gamma[:, None]
    diff = gz * uc_low[0] - ax * uc_low[1]
    om2 = (-diff.imag + 1j * diff.real).astype(np.complex64)
    return {
        "om2": om2,
        "uc_low": uc_low,
        "visc": np.float32(1.0 / float(np.float32(Re))),
        "seed_out": int(seed_out),
        "Q2": mom["Q2"],
        "W2": mom["W2"],
    }
