"""CPU oracle for the palinstrophy pseudo-spectral DNS step.

TEST INFRASTRUCTURE ONLY.  ``palinstrophy_gb300`` never imports this module.
It is used by ``tests/`` (parity checker), ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``.

It restates the reference CPU (NumPy + scipy.fft) path of
``palinstrophy/turbo_simulator.py``, operation for operation:

  step2a   dealias pad + inverse irfft2(norm='forward')   turbo_simulator.py:2020-2034, 1246-1262
  step2b   uu, ww, uw products, rfft2, zero row z=N       turbo_simulator.py:1449-1513, 1276-1297
  step3    gathered nonlinear term, CNAB2, fnm1, inversion turbo_simulator.py:1520-1585, 1731-1771
  rk3      LS-IMEX-RK3 (alpha, beta) stages              turbo_simulator.py:1900-1943
  cflm     max(|u|+|w|) * N/(2 pi)                        turbo_simulator.py:2106-2125
  next_dt  cn = 0.8 + 0.2 cflnum/CFL, dt *= cn            turbo_simulator.py:2127-2167
  driver   run_dns cadence (it=1, it%UPDATE==0, it=STEPS) turbo_simulator.py:2810-2848
  metrics  flow_eddy_metrics, pal_over_ens_kmax2,         turbo_simulator.py:764-810,
           energy_joules, omega-spectrum shell bins       turbo_main.py:1947-1959, 2015-2073,
                                                          turbo_simulator.py:2317-2383

``dtype=np.float64`` is the FP64 oracle (complex128 everywhere, constants in
double).  ``dtype=np.float32`` keeps the reference's float32 casts and
operation order, so that on one machine it reproduces the reference CPU path
bit for bit; it is also the timed CPU baseline ("port").

Arrays use the reference layouts: om2/fnm1 (N, N/2) [z, kx];
uc_full (3, M, M/2+1) [comp, z, kx]; ur_full (3, M, M) [comp, z, x], M = 3N/2.
"""
from __future__ import annotations

import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.fft as spfft

RK3_ALPHA = (8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0)
RK3_BETA = (0.0, -17.0 / 60.0, -5.0 / 12.0)


_POOL = {}


def _rows(S, n, fn):
    """Run fn(slice) over blocks of rows 0..n-1 on S.threads host threads.

    Only elementwise work goes through here: each output element is computed by
    the same NumPy operations whatever the split, so the results are identical
    to one call over all rows (NumPy releases the GIL inside large ufunc calls).
    """
    k = S.threads
    if k <= 1 or n < 64 * k:
        fn(slice(0, n))
        return
    pool = _POOL.get(k)
    if pool is None:
        pool = _POOL[k] = ThreadPoolExecutor(k)
    b = -(-n // k)
    list(pool.map(fn, [slice(i, min(n, i + b)) for i in range(0, n, b)]))


class OracleState:
    """Minimal DnsState twin holding the arrays and scalars one step touches."""

    def __init__(self, N, om2, uc_low, visc, cflnum, dtype=np.float64, workers=None, threads=None):
        if N % 4:
            raise ValueError("N must be a multiple of 4")
        self.rdt = np.dtype(dtype)
        self.cdt = np.dtype(np.complex64 if self.rdt == np.float32 else np.complex128)
        self.f32 = self.rdt == np.float32
        self.N = N
        self.Nh = N // 2
        self.M = 3 * N // 2
        self.NK_full = self.M // 2 + 1
        # pocketfft batches lines differently per worker count; the reference
        # passes min(8, cpu_count) (turbo_simulator.py:912), so the FP32 port
        # is bit-exact with it only at that same count.
        self.workers = workers if workers else min(8, os.cpu_count() or 1)
        # host threads for the elementwise passes (results do not depend on it)
        self.threads = threads if threads else (os.cpu_count() or 1)
        M, Nh = self.M, self.Nh
        self.ur_full = np.zeros((3, M, M), self.rdt)
        self.uc_full = np.zeros((3, M, self.NK_full), self.cdt)
        self.uc_full[0:2, :N, :Nh] = np.asarray(uc_low).astype(self.cdt)
        self.om2 = np.asarray(om2).astype(self.cdt).copy()
        self.fnm1 = np.zeros_like(self.om2)
        self.visc = float(visc)
        self.cflnum = float(cflnum)
        self.t = 0.0
        self.dt = 0.0
        self.cn = 1.0
        self.cnm1 = 0.0
        self.it = 0
        r = self.rdt.type
        alfa = np.arange(Nh, dtype=self.rdt)
        kz = np.arange(N)
        gamma = np.where(kz < Nh, kz, kz - N).astype(self.rdt)
        self.alfa, self.gamma = alfa, gamma
        ax = alfa[None, :]
        gz = gamma[:, None]
        self.K2 = (ax * ax + gz * gz).astype(self.rdt)
        self.GA = (gz * ax).astype(self.rdt)
        self.G2mA2 = (gz * gz - ax * ax).astype(self.rdt)
        self.invK2_sub = (r(1.0) / (self.K2[:, 1:] + r(1.0e-30))).astype(self.rdt)
        mask0 = (kz >= 1) & (np.abs(gamma) > 0.0)
        safe = np.where(mask0, gamma, r(1.0))
        self.inv_gamma0 = (r(1.0) / safe).astype(self.rdt) * mask0.astype(self.rdt)
        m32 = r(1.5) * r(N)
        self.divxz = r(1.0) / (m32 * m32)
        self.inv_dx = float(N) / (2.0 * math.pi)

    # ---------------- scalar helpers ---------------------------------
    def _s(self, v):
        """Scalar in the working precision (float32 cast as in TS:1736-1737)."""
        return self.rdt.type(v)


def step2a(S: OracleState) -> None:
    """Pad the velocity low band to the 3/2 grid and inverse-transform (TS:2020-2034)."""
    N, Nh = S.N, S.Nh
    UC = S.uc_full
    hi_end = min(3 * N // 4, S.NK_full - 1)

    def pad(sl):
        UC[0:2, sl, Nh:hi_end + 1] = 0

    def move(sl):  # rows Nh..N-1 -> N..N+Nh-1 (disjoint ranges), then zero the source
        src = slice(Nh + sl.start, Nh + sl.stop)
        UC[0:2, N + sl.start:N + sl.stop, :Nh] = UC[0:2, src, :Nh]
        UC[0:2, src, :Nh] = 0

    _rows(S, S.M, pad)
    _rows(S, Nh, move)
    ur01 = spfft.irfft2(UC[0:2], axes=(1, 2), overwrite_x=True,
                        workers=S.workers, norm="forward")

    def put(sl):
        S.ur_full[0:2, sl] = ur01[:, sl]

    _rows(S, S.M, put)


def step2b(S: OracleState) -> None:
    """In-place products, forward rfft2 of the 3 planes, zero row z=N (TS:1449-1513)."""
    UR = S.ur_full

    def products(sl):
        u, w = UR[0, sl], UR[1, sl]
        np.multiply(u, w, out=UR[2, sl])
        np.multiply(u, u, out=u)
        np.multiply(w, w, out=w)

    _rows(S, S.M, products)
    S.uc_full = spfft.rfft2(UR, axes=(1, 2), overwrite_x=True, workers=S.workers)
    S.uc_full[0:3, S.N, 0:S.Nh] = 0


def nonlinear(S: OracleState) -> np.ndarray:
    """fn = divxz [GA (F uu - F ww) + (G^2 - A^2) F uw] at gathered rows (TS:1520-1552).

    Output row z < N/2 reads uc_full row z, row z >= N/2 reads row z + N/2."""
    N, Nh = S.N, S.Nh
    UC = S.uc_full
    out = np.empty((N, Nh), S.cdt)

    def blk(sl):
        for lo, hi, off in ((sl.start, min(sl.stop, Nh), 0), (max(sl.start, Nh), sl.stop, Nh)):
            if lo >= hi:
                continue
            o, g = slice(lo, hi), slice(lo + off, hi + off)
            r = np.subtract(UC[0, g, :Nh], UC[1, g, :Nh])
            np.multiply(r, S.GA[o], out=r)
            tmp = np.multiply(UC[2, g, :Nh], S.G2mA2[o])
            np.add(r, tmp, out=r)
            np.multiply(r, S.divxz, out=r)
            out[o] = r

    _rows(S, N, blk)
    return out


def reconstruct_velocity(S: OracleState) -> None:
    """omega -> (u1, u3) low band of uc_full (TS:1555-1585)."""
    N, Nh = S.N, S.Nh
    om = S.om2
    UC = S.uc_full
    mi = S.cdt.type(-1j)
    pi_ = S.cdt.type(1j)

    def blk(sl):
        o = om[sl]
        out1 = np.zeros_like(o)
        out2 = np.zeros_like(o)
        if Nh > 1:
            o1 = o[:, 1:] * S.invK2_sub[sl]
            o1 = o1 * S.gamma[sl, None]
            out1[:, 1:] = o1 * mi
            o2 = o[:, 1:] * S.invK2_sub[sl]
            o2 = o2 * S.alfa[1:][None, :]
            out2[:, 1:] = o2 * pi_
        out1[:, 0] = mi * o[:, 0] * S.inv_gamma0[sl]
        out2[:, 0] = 0
        UC[0, sl, :Nh] = out1
        UC[1, sl, :Nh] = out2

    _rows(S, N, blk)


def step3(S: OracleState) -> None:
    """CNAB2 update with the stale-cn AB2 weights (TS:1731-1771)."""
    s = S._s
    visc, dt, cnm1 = s(S.visc), s(S.dt), s(S.cnm1)
    fn = nonlinear(S)
    vt = s(0.5) * visc * dt
    c2 = s(0.5) * dt * (s(2.0) + cnm1)
    c3 = -s(0.5) * dt * cnm1
    om, fm = S.om2, S.fnm1
    new = np.empty_like(om)

    def blk(sl):
        arg = S.K2[sl] * vt
        den = arg + s(1.0)
        num = om[sl] - om[sl] * arg
        num = num + fn[sl] * c2
        num = num + fm[sl] * c3
        new[sl] = num / den

    _rows(S, S.N, blk)
    S.om2 = new
    S.fnm1 = fn
    reconstruct_velocity(S)
    S.cnm1 = float(S.cn)


def rk3(S: OracleState) -> None:
    """One LS-IMEX-RK3 step: 3 x (step2b, stage update, step2a) (TS:1900-1943)."""
    s = S._s
    dt, visc = s(S.dt), s(S.visc)
    for a_, b_ in zip(RK3_ALPHA, RK3_BETA):
        a, b = s(a_), s(b_)
        step2b(S)
        fn = nonlinear(S)
        kb, fa, fb, ka = b * dt * visc, a * dt, b * dt, a * dt * visc
        om, fm = S.om2, S.fnm1
        new = np.empty_like(om)

        def blk(sl):
            rhs = s(1.0) - S.K2[sl] * kb
            num = om[sl] * rhs
            num = num + fn[sl] * fa
            num = num + fm[sl] * fb
            den = S.K2[sl] * ka + s(1.0)
            new[sl] = num / den

        _rows(S, S.N, blk)
        S.om2 = new
        S.fnm1 = fn
        reconstruct_velocity(S)
        step2a(S)


def cnab2(S: OracleState) -> None:
    step2b(S)
    step3(S)
    step2a(S)


def compute_cflm(S: OracleState) -> float:
    """max(|u|+|w|) * N/(2 pi) over the 3/2 grid (TS:2106-2125)."""
    tmp = np.abs(S.ur_full[0]) + np.abs(S.ur_full[1])
    return float(tmp.max() * S.inv_dx)


def next_dt(S: OracleState) -> float:
    """CFL-adaptive dt update in double (TS:2160-2167)."""
    cflm = compute_cflm(S)
    if cflm <= 0.0 or S.dt <= 0.0:
        return cflm
    cfl = cflm * S.dt * math.pi
    S.cn = 0.8 + 0.2 * (S.cflnum / cfl)
    S.dt = S.dt * S.cn
    return cflm


def init_dt(S: OracleState) -> float:
    """Initial step2a + dt = cflnum/(CFLM pi), cn=1, cnm1=0 (TS:2810-2823)."""
    step2a(S)
    cflm = compute_cflm(S)
    S.dt = S.cflnum / (cflm * math.pi)
    S.cn, S.cnm1, S.t = 1.0, 0.0, 0.0
    return cflm


def run(S: OracleState, steps: int, method: str = "CNAB2", update: int = 100,
        dt_replay=None, log=None) -> None:
    """The run_dns hot loop (TS:2831-2848).

    ``dt_replay``: optional sequence of (dt, cn) pairs, one per next_dt call, that
    replaces the computed values (the reference's dt sequence replayed).
    ``log``: optional list receiving (it, t, dt, cn, cflm) at each next_dt.
    """
    step = rk3 if method.upper() == "LS_IMEX_RK3" else cnab2
    nd = 0
    for it in range(1, steps + 1):
        S.it = it
        dt_old = S.dt
        step(S)
        if it % update == 0 or it == 1 or it == steps:
            cflm = next_dt(S)
            if dt_replay is not None:
                S.dt, S.cn = float(dt_replay[nd][0]), float(dt_replay[nd][1])
            nd += 1
            if log is not None:
                log.append((it, S.t, S.dt, S.cn, cflm))
        S.t += dt_old


# ---------------- diagnostics ---------------------------------------
def rfft_weights(nh: int, last_one: bool = True) -> np.ndarray:
    """[1,2,...,2,1] as the eddy/pal metrics use it (TS:778-781, TM:2040-2044)."""
    w = np.full(nh, 2.0)
    w[0] = 1.0
    if last_one and nh > 1:
        w[-1] = 1.0
    return w


def flow_eddy_metrics(S: OracleState):
    """(U, L, tau_L) in double from ur_full and om2 (TS:764-810)."""
    u, v = S.ur_full[0].astype(np.float64), S.ur_full[1].astype(np.float64)
    U = math.sqrt(max(0.0, float(np.mean(u * u + v * v))))
    K2 = S.K2.astype(np.float64)
    p = np.abs(S.om2.astype(np.complex128)) ** 2
    power = np.where(K2 > 0, p / np.where(K2 > 0, K2, 1.0), 0.0)
    wp = power * rfft_weights(S.Nh)[None, :]
    e = float(wp.sum() - wp[0, 0])
    if e <= 0.0:
        return U, float("nan"), float("nan")
    invk = np.where(K2 > 0, 1.0 / np.sqrt(np.where(K2 > 0, K2, 1.0)), 0.0)
    L = 2.0 * math.pi * float((wp * invk).sum()) / e
    return U, L, (L / U if U > 0 else float("nan"))


def spectral_sums(S: OracleState) -> dict:
    """E, Z (enstrophy), P (palinstrophy), kmax^2 and the GUI ratio (TM:2015-2073)."""
    K2 = S.K2.astype(np.float64)
    p = np.abs(S.om2.astype(np.complex128)) ** 2
    w = rfft_weights(S.Nh)[None, :]
    wp = w * p
    Z = float(wp.sum() - p[0, 0])
    kmax2 = float(K2.max())
    P = float((w * K2 * p).sum())
    power = np.where(K2 > 0, p / np.where(K2 > 0, K2, 1.0), 0.0)
    E = float((power * w).sum())
    ratio = P / (Z * kmax2) if Z > 0 and kmax2 > 0 else 0.0
    return {"E": E, "Z": Z, "P": P, "kmax2": kmax2, "pal_over_ens_kmax2": ratio}


def energy_joules(S: OracleState) -> float:
    """0.5 (2 pi)^2 <u^2+v^2> on the 3/2 grid (TM:1947-1959)."""
    u, v = S.ur_full[0].astype(np.float64), S.ur_full[1].astype(np.float64)
    return 0.5 * (2.0 * math.pi) ** 2 * float((u * u).sum() + (v * v).sum()) / u.size


def omega_spectrum_bins(S: OracleState):
    """Shell sums of |omega|^2/k^2 (weight 2 for kx>0) -- TS:2317-2383."""
    n = S.N
    nbins = max(32, 2 * n)
    r_max = math.sqrt(2.0)
    k_nyq = 0.5 * n
    scale2 = float(S.M * S.M) ** 2
    om = S.om2.astype(np.complex128)
    kx = np.arange(S.Nh, dtype=np.float64)
    wt = np.ones(S.Nh)
    wt[1:] = 2.0
    esum = np.zeros(nbins)
    cnt = np.zeros(nbins, dtype=np.int64)
    for z in range(n):
        kz = z if z < n // 2 else z - n
        k2 = kx * kx + float(kz * kz)
        m = k2 > 0
        b = np.floor((np.sqrt(k2[m]) / k_nyq / r_max) * nbins).astype(np.int64)
        np.clip(b, 0, nbins - 1, out=b)
        p = (om[z, m].real ** 2 + om[z, m].imag ** 2) / k2[m]
        esum += np.bincount(b, weights=p * wt[m] * scale2, minlength=nbins)
        cnt += np.bincount(b, weights=wt[m], minlength=nbins).astype(np.int64)
    return esum, cnt


def rel_l2(ref, cand) -> float:
    ref = np.asarray(ref).astype(np.complex128)
    cand = np.asarray(cand).astype(np.complex128)
    return float(np.linalg.norm((cand - ref).ravel()) / max(np.linalg.norm(ref.ravel()), 1e-300))


# ---------------- display fields (turbo_simulator.py:2629-2708) -------------
def band_to_phys(S: OracleState, band) -> np.ndarray:
    """Pad a compact (N, N/2) band like STEP2A, zero the kz=-N/2 row, irfft2."""
    N, Nh, M = S.N, S.Nh, S.M
    tmp = np.zeros((M, S.NK_full), S.cdt)
    tmp[:N, :Nh] = band
    tmp[:, Nh:min(3 * N // 4, S.NK_full - 1) + 1] = 0
    tmp[N:N + Nh, :Nh] = tmp[Nh:N, :Nh]
    tmp[Nh:N, :Nh] = 0
    tmp[N, :Nh] = 0
    return spfft.irfft2(tmp, s=(M, M), axes=(0, 1), norm="forward", workers=S.workers)


def om2_phys(S: OracleState) -> np.ndarray:
    return band_to_phys(S, S.om2)


def stream_func(S: OracleState) -> np.ndarray:
    K2 = S.K2 + S.rdt.type(1.0e-30)
    return band_to_phys(S, S.om2 / K2)


def kinetic(S: OracleState) -> np.ndarray:
    u, w = S.ur_full[0], S.ur_full[1]
    return np.sqrt(u * u + w * w)


def to_pixels(field) -> np.ndarray:
    """8-bit frame as turbo_wrapper.py:317-351 (1..255, 128 if constant)."""
    f = np.asarray(field, np.float64)
    lo, hi = f.min(), f.max()
    if abs(hi - lo) <= 1e-12:
        return np.full(f.shape, 128, np.uint8)
    return np.clip(1.0 + (f - lo) / (hi - lo) * 254.0, 1.0, 255.0).astype(np.uint8)
