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


def _lcg_draws(N, seed):
    """The serial LCG + shuffle draws of the PAO loop (turbo_simulator.py:241-286),
    in the reference's call order, as the float32 variates v[z, x]; plus the final
    seed.  Every state after the first step lies in 0..ID-1, so the next state and
    the shuffle slot of each state are looked up from tables."""
    nh = N // 2
    r_of = (np.arange(LCG_ID, dtype=np.float32) / np.float32(LCG_ID)).astype(np.float32)
    nxt = [(s * LCG_IMM + LCG_IT) % LCG_ID for s in range(LCG_ID)]
    slot = [min(max(int(float(r) * 97.0), 0), 96) for r in r_of.tolist()]
    s = int(seed)
    for _ in range(97):
        s = (s * LCG_IMM + LCG_IT) % LCG_ID
    table = []
    for _ in range(97):
        s = nxt[s]
        table.append(s)
    out = [0] * (N * nh)
    for i in range(N * nh):
        s = nxt[s]
        k = slot[s]
        out[i] = table[k]
        table[k] = s
    return r_of[np.asarray(out, dtype=np.int64)].reshape(N, nh), s


def _hash01_vec(x, z, seed, salt):
    """hash01 over arrays of mode indices: the affine argument in NumPy float64
    (the same IEEE operations in the same order), sin from the math module."""
    a = (x.astype(np.float64) + 1.0) * 12.9898 + (z.astype(np.float64) + 1.0) * 78.233
    a = a + (float(seed) + 1.0) * 0.010001
    a = a + (float(salt) + 1.0) * 37.719
    s = np.array([math.sin(v) for v in a.tolist()], dtype=np.float64) * 43758.5453123
    return s - np.floor(s)


def _c64_scale(a, pr, pi):
    """complex64(a) * (pr + i pi) as two float32 planes, with NumPy scalar
    complex64 multiplication's textbook formula (each product rounded alone)."""
    zero = np.float32(0.0)
    return a * pr - zero * pi, a * pi + zero * pr


def _c64(re, im):
    """complex64 array from float32 planes, keeping the signs of zeros."""
    out = np.empty(np.shape(re), np.complex64)
    out.real = re
    out.imag = im
    return out


def generate_fast(N: int, K0: float, Re: float, seed: int, spectrum: str = "KM3"):
    """The arrays of generate() with the per-mode work vectorised (seconds at
    N=4096 instead of minutes).  The LCG stays serial; float32 values come from
    the same NumPy float32 operations; the double shell and moment sums keep the
    reference's serial order (np.add.at and np.add.accumulate add in index order).
    Checked against generate() and the reference fixtures in the tests."""
    if N % 4 or N < 8:
        raise ValueError("N must be a multiple of 4 and >= 8")
    spectrum = spectrum.upper()
    if spectrum not in ("KM3", "PAO"):
        raise ValueError(f"unknown start spectrum {spectrum!r}")
    km3 = spectrum == "KM3"
    nh = N // 2
    alfa, gamma = wavenumbers(N)
    k0 = np.float32(K0)
    v, seed_out = _lcg_draws(N, int(seed))                     # [z, x]
    th = (np.float32(2.0) * PI32) * v
    c, s = np.cos(th), np.sin(th)
    ax = alfa[None, :]
    gz = gamma[:, None]
    k2 = gz * gz + ax * ax
    k = np.sqrt(k2)
    e = np.exp(-(k / k0) * (k / k0))
    norm = PI32 * k0 * k0
    zero_x = np.broadcast_to(ax == 0.0, (N, nh))
    with np.errstate(divide="ignore", invalid="ignore"):
        den = np.float32(1.0) + (gz * gz) / (ax * ax)
        e2 = np.where(zero_x, e / norm, e / (den * norm)).astype(np.float32)
    if km3:
        e2 = np.where(e2 < np.float32(1.0e-40), np.float32(1.0e-40), e2)
    amp = np.sqrt(e2)
    wr, wi = _c64_scale(amp, c, s)
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.where(zero_x, np.float32(0.0), -(gz / ax)).astype(np.float32)
    ur_r, ur_i = _c64_scale(ratio, wr, wi)
    # UR[x, z, comp] as complex64 planes, comp 0 = u1, 1 = u3
    w = _c64(wr, wi)
    u1 = np.where(zero_x, w, _c64(ur_r, ur_i)).T.copy()
    u3 = np.where(zero_x, np.complex64(0), w).T.copy()
    u1[0, 0] = u3[0, 0] = 0
    zz = np.arange(1, nh)
    u1[0, N - zz] = np.conj(u1[0, zz])
    u3[0, N - zz] = np.conj(u3[0, zz])
    u1[:, nh] = 0
    u3[:, nh] = 0
    xs = np.repeat(np.arange(nh), N)                            # x-major order
    zs = np.tile(np.arange(N), nh)
    m = np.where(xs == 0, 1.0, 2.0)
    ax2 = alfa.astype(np.float64)[xs] ** 2
    gz2 = gamma.astype(np.float64)[zs] ** 2
    if km3:
        knyq = float(nh)
        kd = np.sqrt(ax2 + gz2)
        sh = (kd + 0.5).astype(np.int64)
        keep = (kd > 0.0) & (kd <= knyq) & (sh <= nh)
        f1, f3 = u1.ravel(), u3.ravel()

        def pw(f):
            re, im = f.real.astype(np.float64), f.imag.astype(np.float64)
            return re * re + im * im

        e_shell = np.zeros(nh + 1)
        w_shell = np.zeros(nh + 1)
        np.add.at(e_shell, sh[keep], (m * (pw(f1) + pw(f3)))[keep])
        zh = np.where((xs == 0) & (zs > nh), N - zs, zs)
        jit = 0.75 + 0.50 * _hash01_vec(xs[keep], zh[keep], seed, 17)
        np.add.at(w_shell, sh[keep], m[keep] * jit)
        kk0 = max(float(k0), 1.0)
        target = np.zeros(nh + 1)
        for q in range(1, nh + 1):
            kq = float(q)
            if kq < kk0:
                lo = kq / kk0
                target[q] = (lo * lo * lo * lo) / (kk0 * kk0 * kk0)
            else:
                target[q] = 1.0 / (kq * kq * kq)
        e_orig = e_target = 0.0
        for q in range(1, nh + 1):
            e_orig += e_shell[q]
            e_target += target[q]
        if e_orig > 0.0 and e_target > 0.0:
            scale = e_orig / e_target
            sel = keep & (w_shell[np.minimum(sh, nh)] > 0.0)
            new1 = np.zeros(nh * N, np.complex64)
            new3 = np.zeros(nh * N, np.complex64)
            xi, zi, si = xs[sel], zs[sel], sh[sel]
            neg = (xi == 0) & (zi > nh)
            zhs = np.where(neg, N - zi, zi)
            sign = np.where(neg, -1.0, 1.0)
            jit = 0.75 + 0.50 * _hash01_vec(xi, zhs, seed, 17)
            e_mode = (scale * target[si]) * jit / w_shell[si]
            thd = sign * 2.0 * math.pi * _hash01_vec(xi, zhs, seed, 53)
            tl = thd.tolist()
            pr = np.array([math.cos(t) for t in tl], dtype=np.float64).astype(np.float32)
            pim = np.array([math.sin(t) for t in tl], dtype=np.float64).astype(np.float32)
            axs = alfa.astype(np.float64)[xi]
            gzs = gamma.astype(np.float64)[zi]
            z0 = axs == 0.0
            with np.errstate(divide="ignore", invalid="ignore"):
                a_w = np.where(z0, np.sqrt(e_mode), np.sqrt(e_mode / (1.0 + gzs * gzs / (axs * axs))))
                rat = np.where(z0, 0.0, -gzs / axs).astype(np.float32)
            wr, wi = _c64_scale(a_w.astype(np.float32), pr, pim)
            qr, qi = _c64_scale(rat, wr, wi)
            w = _c64(wr, wi)
            q = _c64(qr, qi)
            idx = xi * N + zi
            new1[idx] = np.where(z0, w, q)
            new3[idx] = np.where(z0, np.complex64(0), w)
            u1 = new1.reshape(nh, N)
            u3 = new3.reshape(nh, N)
    f1, f3 = u1.ravel(), u3.ravel()
    p1 = f1.real.astype(np.float64) ** 2 + f1.imag.astype(np.float64) ** 2
    p3 = f3.real.astype(np.float64) ** 2 + f3.imag.astype(np.float64) ** 2

    def serial(t):
        return float(np.add.accumulate(t)[-1])

    a1, a2 = serial(m * p1), serial(m * p3)
    a3, a4 = serial(m * p1 * ax2), serial(m * p1 * gz2)
    a5, a6 = serial(m * p3 * ax2), serial(m * p3 * gz2)
    uc_low = np.ascontiguousarray(np.stack([u1.T, u3.T]))     # (2, N, N/2)
    diff = gz * uc_low[0] - ax * uc_low[1]
    om2 = (-diff.imag + 1j * diff.real).astype(np.complex64)
    return {"om2": om2, "uc_low": uc_low, "visc": np.float32(1.0 / float(np.float32(Re))),
            "seed_out": int(seed_out), "Q2": a1 + a2, "W2": a3 + a4 + a5 + a6}
