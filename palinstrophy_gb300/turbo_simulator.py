"""Drop-in GB300 backend for palinstrophy's DNS stepping/initialisation API.

The names, signatures and DnsState fields mirror
``palinstrophy/turbo_simulator.py`` so that its callers (``run_dns``, the
``turbo_wrapper.DnsSimulator`` facade and the GUI) run unchanged with
``backend="gb300"``:

  create_dns_state      turbo_simulator.py:878-1054
  dns_step2a            turbo_simulator.py:1949-2100
  dns_step2b            turbo_simulator.py:1378-1513
  dns_step3             turbo_simulator.py:1588-1771
  dns_step_ls_imex_rk3  turbo_simulator.py:1900-1943
  compute_cflm          turbo_simulator.py:2106-2125
  next_dt               turbo_simulator.py:2127-2167
  sync_time_scalars_from_device  turbo_simulator.py:846-854
  DnsState.flow_eddy_metrics     turbo_simulator.py:764-810
  run_dns / compare_time_steppers turbo_simulator.py:2744-2903

Every step runs in the hand-written sm_103a kernels of libpalgpu.so; there is
no CPU path here.  om2 and fnm1 are host NumPy copies taken on access, as the
reference GUI does with cp.asnumpy at frame pulls; ur_full is a persistent host
array whose velocity planes refresh from the device when read after a step and
whose third plane holds the display helpers' output, as in the reference.
"""
from __future__ import annotations

import math
import os
import sys
import time
from typing import Literal

import numpy as np

from . import _lib as L

SCIPYTURBO_SEED_ENV = "SCIPYTURBO_SEED"
PAO_SEED_MIN = 1
PAO_SEED_MAX = 5010
TimeStepper = Literal["CNAB2", "LS_IMEX_RK3", "CHECK"]
SPECTRUM = Literal["PAO", "KM3"]
_METHODS = {"CNAB2": L.PAL_CNAB2, "LS_IMEX_RK3": L.PAL_LS_IMEX_RK3}
_PREC = {"fp32": L.PAL_FP32, "fp64": L.PAL_FP64}


def pao_seed_from_env(default: int | None = None) -> int | None:
    """Seed from $SCIPYTURBO_SEED, validated to 1..5010 (turbo_simulator.py:54-73)."""
    raw = os.environ.get(SCIPYTURBO_SEED_ENV)
    if raw is None or raw.strip() == "":
        return default
    try:
        seed = int(raw.strip(), 10)
    except ValueError as exc:
        raise ValueError(f"{SCIPYTURBO_SEED_ENV} must be an integer from {PAO_SEED_MIN} to "
                         f"{PAO_SEED_MAX}; got {raw!r}") from exc
    if not PAO_SEED_MIN <= seed <= PAO_SEED_MAX:
        raise ValueError(f"{SCIPYTURBO_SEED_ENV} must be from {PAO_SEED_MIN} to {PAO_SEED_MAX}; got {seed}")
    return seed


class Field:
    """One N x N field on the GPU: owns a pal_handle and its device state."""

    def __init__(self, N: int, precision: str = "fp32", Re: float = 1e4, cfl: float = 0.75):
        if precision not in _PREC:
            raise ValueError("precision must be 'fp32' or 'fp64'")
        self.lib = L.load()
        self.N = int(N)
        self.M = 3 * self.N // 2
        self.precision = precision
        self.cdt = np.complex64 if precision == "fp32" else np.complex128
        self.rdt = np.float32 if precision == "fp32" else np.float64
        h = L._H()
        L.check(self.lib.pal_create(self.N, _PREC[precision], float(Re), float(cfl), h))
        self.h = h
        # bumped by every call that changes the field, so host copies know when they are stale
        self.gen = 0

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.pal_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        return L.check(rc, self.h)

    # -- state ------------------------------------------------------------
    def set_state_device(self, om2_ptr: int):
        """om2 from device memory: a C-contiguous (N, N/2) array of the handle's
        complex type at om2_ptr (fnm1 = 0, velocity from the om2 inversion)."""
        self.gen += 1
        self._ck(self.lib.pal_set_spectral_state(self.h, L.ctypes.c_void_p(int(om2_ptr)), None))

    def set_state(self, om2, fnm1=None, uc_low=None):
        self.gen += 1
        om2 = np.ascontiguousarray(om2, dtype=self.cdt)
        if om2.shape != (self.N, self.N // 2):
            raise ValueError(f"om2 must have shape {(self.N, self.N // 2)}")
        f = None if fnm1 is None else np.ascontiguousarray(fnm1, dtype=self.cdt)
        self._ck(self.lib.pal_set_spectral_state(self.h, L.ptr(om2), None if f is None else L.ptr(f)))
        if uc_low is not None:
            uc = np.ascontiguousarray(uc_low, dtype=self.cdt)
            if uc.shape != (2, self.N, self.N // 2):
                raise ValueError(f"uc_low must have shape {(2, self.N, self.N // 2)}")
            self._ck(self.lib.pal_set_velocity_spectrum(self.h, L.ptr(uc)))

    def generate(self, K0: float, Re: float, seed: int, spectrum: str = "KM3"):
        """PAO / KM3 start generated on the device (pal_generate); returns
        (uc_low (2, N, N/2) host copy, stats dict as pao_generate's)."""
        self.gen += 1
        spec = {"KM3": L.PAL_SPEC_KM3, "PAO": L.PAL_SPEC_PAO}[spectrum.upper()]
        uc = np.empty((2, self.N, self.N // 2), self.cdt)
        st = (L._D * 3)()
        so = L.ctypes.c_int(0)
        self._ck(self.lib.pal_generate(self.h, float(K0), float(Re), int(seed), spec, L.ptr(uc), st,
                                       L.ctypes.byref(so)))
        return uc, {"Energy": st[0], "WiWi": st[1], "visc": st[2], "seed_out": so.value}

    def set_scalars(self, t=0.0, dt=0.0, cn=1.0, cnm1=0.0, visc=1e-4, cflnum=0.75, it=0):
        self._ck(self.lib.pal_set_scalars(self.h, t, dt, cn, cnm1, visc, cflnum, int(it)))

    def set_scalar(self, which: str, value):
        idx = {"t": L.PAL_SC_T, "dt": L.PAL_SC_DT, "cn": L.PAL_SC_CN, "cnm1": L.PAL_SC_CNM1,
               "visc": L.PAL_SC_VISC, "cflnum": L.PAL_SC_CFLNUM, "it": L.PAL_SC_IT}[which]
        self._ck(self.lib.pal_set_scalar(self.h, idx, float(value)))

    def scalars(self) -> dict:
        v = [L._D() for _ in range(6)]
        it = L.ctypes.c_longlong()
        self._ck(self.lib.pal_get_scalars(self.h, *[L.ctypes.byref(x) for x in v], L.ctypes.byref(it)))
        return dict(zip(("t", "dt", "cn", "cnm1", "visc", "cflnum"), [x.value for x in v]), it=it.value)

    # -- stepping -----------------------------------------------------------
    def step2a(self):
        self.gen += 1
        self._ck(self.lib.pal_step2a(self.h))

    def step2b(self):
        self.gen += 1
        self._ck(self.lib.pal_step2b(self.h))

    def step3(self):
        self.gen += 1
        self._ck(self.lib.pal_step3(self.h))

    def step_rk3(self):
        self.gen += 1
        self._ck(self.lib.pal_step_rk3(self.h))

    def step(self, method="CNAB2", nsteps=1, update=0, final_update=False):
        self.gen += 1
        self._ck(self.lib.pal_step(self.h, _METHODS[method], int(nsteps), int(update), int(bool(final_update))))

    def compute_cflm(self) -> float:
        c = L._D()
        self._ck(self.lib.pal_compute_cflm(self.h, L.ctypes.byref(c)))
        return c.value

    def next_dt(self, sync_host=True):
        c = L._D()
        self._ck(self.lib.pal_next_dt(self.h, int(bool(sync_host)), L.ctypes.byref(c)))
        return c.value if sync_host else None

    def diagnostics(self) -> dict:
        d = L.PalDiag()
        rc = self.lib.pal_diagnostics(self.h, L.ctypes.byref(d))
        out = {n: getattr(d, n) for n, _ in L.PalDiag._fields_}
        if rc == L.PAL_ERR_NONFINITE:
            return out
        self._ck(rc)
        return out

    def synchronize(self):
        self._ck(self.lib.pal_synchronize(self.h))

    def profile_kernels(self, method="LS_IMEX_RK3", nsteps=5):
        """Average k_row / k_col launch durations (ms) from events on the handle stream."""
        r, c, n = L._D(), L._D(), L._I()
        self._ck(self.lib.pal_profile_kernels(self.h, _METHODS[method], int(nsteps), L.ctypes.byref(r),
                                              L.ctypes.byref(c), L.ctypes.byref(n)))
        return r.value, c.value, n.value

    def variant(self) -> dict:
        """The kernel candidates the autotuner selected for this size."""
        r, c, nr, nc = L._I(), L._I(), L._I(), L._I()
        buf = L.ctypes.create_string_buffer(256)
        self._ck(self.lib.pal_get_variant(self.h, L.ctypes.byref(r), L.ctypes.byref(c), L.ctypes.byref(nr),
                                          L.ctypes.byref(nc), buf, len(buf)))
        rb, cb = L._I(), L._I()
        self._ck(self.lib.pal_get_occupancy(self.h, L.ctypes.byref(rb), L.ctypes.byref(cb)))
        return {"row": r.value, "col": c.value, "n_rows": nr.value, "n_cols": nc.value,
                "desc": buf.value.decode(), "row_blocks_per_sm": rb.value, "col_blocks_per_sm": cb.value}

    def set_variant(self, row: int, col: int):
        self._ck(self.lib.pal_set_variant(self.h, int(row), int(col)))

    def set_debug(self, what: int, value: int):
        """Test switch (pal_set_debug), e.g. L.PAL_DBG_SKIP_FIRST_WAIT."""
        self._ck(self.lib.pal_set_debug(self.h, int(what), int(value)))

    def stream_ptr(self) -> int:
        p = L._P()
        self._ck(self.lib.pal_get_stream(self.h, L.ctypes.byref(p)))
        return p.value

    # -- fields -------------------------------------------------------------
    def om2(self):
        a = np.empty((self.N, self.N // 2), self.cdt)
        self._ck(self.lib.pal_get_field(self.h, L.PAL_FIELD_OM2, L.ptr(a)))
        return a

    def fnm1(self):
        a = np.empty((self.N, self.N // 2), self.cdt)
        self._ck(self.lib.pal_get_field(self.h, L.PAL_FIELD_FNM1, L.ptr(a)))
        return a

    def ur(self, comp: int):
        a = np.empty((self.M, self.M), self.rdt)
        return self.ur_into(comp, a)

    def ur_into(self, comp: int, out):
        """Physical u (comp 0) or v (1) into a C-contiguous (M, M) host array."""
        if out.shape != (self.M, self.M) or out.dtype != self.rdt or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous ({self.M}, {self.M}) {np.dtype(self.rdt).name} array")
        self._ck(self.lib.pal_get_field(self.h, L.PAL_FIELD_UR_U if comp == 0 else L.PAL_FIELD_UR_V, L.ptr(out)))
        return out

    def adjoint_palinstrophy(self, nsteps: int, ckpt_every: int = 20):
        """(L, dL/d om2) for L = final palinstrophy after nsteps fixed-dt RK3 steps."""
        self.gen += 1
        g = np.empty((self.N, self.N // 2), self.cdt)
        loss = L._D()
        self._ck(self.lib.pal_adjoint_palinstrophy(self.h, int(nsteps), int(ckpt_every), L.ctypes.byref(loss),
                                                   L.ptr(g)))
        return loss.value, g

    def vis(self, var: int, field: bool = True, pixels: bool = False, out=None):
        """Display field var (VAR_U..VAR_STREAM): (float field or None, uint8 pixels or None);
        `out`, a C-contiguous (M, M) array of the handle's real type, receives the field."""
        if out is not None and (out.shape != (self.M, self.M) or out.dtype != self.rdt
                                or not out.flags.c_contiguous):
            raise ValueError(f"out must be a C-contiguous ({self.M}, {self.M}) {np.dtype(self.rdt).name} array")
        f = out if out is not None else (np.empty((self.M, self.M), self.rdt) if field else None)
        p = np.empty((self.M, self.M), np.uint8) if pixels else None
        self._ck(self.lib.pal_vis_field(self.h, int(var), None if f is None else L.ptr(f),
                                        None if p is None else p.ctypes.data_as(L.ctypes.POINTER(L.ctypes.c_ubyte))))
        return f, p

    def energy_spectrum(self, nbins: int, r_max: float, k_nyq: float):
        e = np.zeros(nbins, np.float64)
        c = np.zeros(nbins, np.int32)
        self._ck(self.lib.pal_energy_spectrum(self.h, int(nbins), float(r_max), float(k_nyq),
                                              e.ctypes.data_as(L._DP), c.ctypes.data_as(L.ctypes.POINTER(L._I))))
        return e, c

    def device_ptr(self, which: int) -> int:
        p = L._P()
        self._ck(self.lib.pal_field_device_ptr(self.h, which, L.ctypes.byref(p)))
        return p.value

    def device_array(self, which: str):
        """Zero-copy device view of a field, with __cuda_array_interface__ (v3):
        "om2" / "fnm1" as the reference's (N, N/2) array (the device keeps them
        [kx][z], so the view is strided), "u" / "v" as the physical (M, M)
        planes (materialised first).  Valid until the handle's next call that
        writes the field; synchronise the handle's stream before reading."""
        idx = {"om2": L.PAL_FIELD_OM2, "fnm1": L.PAL_FIELD_FNM1, "u": L.PAL_FIELD_UR_U, "v": L.PAL_FIELD_UR_V}[which]
        if which in ("u", "v"):
            self._ck(self.lib.pal_materialize_physical(self.h))
        ptr = self.device_ptr(idx)
        esz = np.dtype(self.cdt).itemsize
        if which in ("om2", "fnm1"):
            N = self.N
            return _DeviceView(ptr, (N, N // 2), np.dtype(self.cdt).str, (esz, N * esz), self)
        M = 3 * self.N // 2
        rsz = esz // 2
        return _DeviceView(ptr, (M, M), np.dtype(self.cdt).type(0).real.dtype.str, (M * rsz, rsz), self)


class _DeviceView:
    """A device array exposed through __cuda_array_interface__ (version 3); it
    keeps its handle alive."""

    def __init__(self, ptr, shape, typestr, strides, owner):
        self._owner = owner
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "strides": tuple(strides), "version": 3, "stream": None}


class _UrFull:
    """`DnsState.ur_full`, the (3, M, M) physical planes of the reference state.

    A persistent host array: plane 0 (u) and plane 1 (v) are copied from the
    device when read after the field changed (per plane, so reading one plane
    moves one plane), and plane 2 keeps what the display helpers -- or the
    caller -- last wrote into it, as the reference's dns_kinetic, dns_om2_phys
    and dns_stream_func leave their result in ur_full[2]
    (turbo_simulator.py:2629-2711) for DnsSimulator.make_pixels_component to
    read (turbo_wrapper.py:436-470).  Indexing returns views of the persistent
    array, refreshed in place; host writes into planes 0 and 1 are not sent to
    the device and last until the field next changes.
    """

    def __init__(self, field):
        self._f = field
        self._a = np.zeros((3, field.M, field.M), field.rdt)
        self._gen = [-1, -1]
        self.shape, self.dtype, self.ndim, self.size = self._a.shape, self._a.dtype, 3, self._a.size

    def _planes(self, key):
        k = key[0] if isinstance(key, tuple) and key else key
        if isinstance(k, (int, np.integer)):
            return [int(k) % 3]
        if isinstance(k, slice):
            return list(range(3))[k]
        return [0, 1, 2]

    def _refresh(self, planes):
        g = self._f.gen
        for p in planes:
            if p < 2 and self._gen[p] != g:
                self._f.ur_into(p, self._a[p])
                self._gen[p] = g

    def plane2(self):
        """The persistent plane 2 (the display helpers' output buffer)."""
        return self._a[2]

    def __getitem__(self, key):
        self._refresh(self._planes(key))
        return self._a[key]

    def __setitem__(self, key, value):
        self._refresh(self._planes(key))
        self._a[key] = value

    def __array__(self, dtype=None, copy=None):
        self._refresh([0, 1])
        return self._a if dtype is None else self._a.astype(dtype)

    def __len__(self):
        return 3


class DnsState:
    """GB300 twin of the reference DnsState (turbo_simulator.py:654-810).

    Scalars dt/cn/cnm1 are host mirrors of device values: assigning them writes
    through to the device (turbo_simulator.py:742-753) and
    sync_time_scalars_from_device refreshes them; visc and cflnum (changed at
    run time by the GUI) write through as well.
    """

    _MIRRORED = {"dt", "cn", "cnm1", "visc", "cflnum"}

    def __init__(self, N, Re, K0, CFL, seed, start_spectrum, precision, populate_compact_ur):
        object.__setattr__(self, "_field", None)
        self.backend = "gb300"
        self.xp = np
        self.precision = precision
        self.Nbase = self.NX = self.NZ = int(N)
        self.NX_full = self.NZ_full = 3 * self.NX // 2
        self.NK_full = self.NX_full // 2 + 1
        self.NK = 3 * self.NX // 4 + 1
        self.Re = Re
        self.K0 = K0
        self.start_spectrum = start_spectrum
        self.seed_init = int(seed)
        self.populate_compact_ur = populate_compact_ur
        self.uc_init = None  # initial velocity low band (2, N, N/2), kept for `uc`
        self.fft_workers = 1
        self.inv_dx = float(N) / (2.0 * math.pi)
        self.t = 0.0
        self.it = 0
        nh = self.NX // 2
        self.alfa = np.arange(nh, dtype=np.float32)
        kz = np.arange(self.NZ)
        self.gamma = np.where(kz < nh, kz, kz - self.NZ).astype(np.float32)
        self.step3_K2 = (self.alfa[None, :] ** 2 + self.gamma[:, None] ** 2).astype(np.float32)
        f = Field(N, precision, Re, CFL)
        object.__setattr__(self, "_field", f)
        object.__setattr__(self, "_ur", _UrFull(f))
        object.__setattr__(self, "visc", float(np.float32(1.0 / float(np.float32(Re)))))
        object.__setattr__(self, "cflnum", float(CFL))
        object.__setattr__(self, "dt", 0.0)
        object.__setattr__(self, "cn", 1.0)
        object.__setattr__(self, "cnm1", 0.0)

    def __setattr__(self, name, value):
        object.__setattr__(self, name, value)
        f = self.__dict__.get("_field")
        if f is not None and name in self._MIRRORED:
            f.set_scalar(name, float(value))

    @property
    def field(self) -> Field:
        return self._field

    def sync(self):
        self._field.synchronize()

    # -- array views (host copies) -----------------------------------------
    @property
    def om2(self):
        return self._field.om2()

    @property
    def fnm1(self):
        return self._field.fnm1()

    @property
    def om2_device(self):
        """om2 as a zero-copy device view (reference shape (N, N/2), strided)."""
        return self._field.device_array("om2")

    def ur_device(self, comp: int):
        """Physical velocity component 0 (u) or 1 (v) as a zero-copy (M, M) device view."""
        return self._field.device_array("u" if comp == 0 else "v")

    @property
    def ur_full(self):
        """(3, M, M): u, v and the display plane (see _UrFull)."""
        return self._ur

    @property
    def ur(self):
        n, m = self.NX, self.NX_full
        off = (m - n) // 2
        full = self.ur_full
        out = np.zeros((n, n, 3), full.dtype)
        out[:, :, 0] = full[0, off:off + n, off:off + n]
        out[:, :, 1] = full[1, off:off + n, off:off + n]
        return out

    @property
    def uc(self):
        """Compact velocity spectrum (N, 3N/4+1, 3) as the reference keeps it: the
        generator's initial velocity, never updated by stepping (turbo_simulator.py:944, 1221)."""
        from .restart import uc_from_low_band
        low = self.uc_init if self.uc_init is not None else np.zeros((2, self.NZ, self.NX // 2), np.complex64)
        return uc_from_low_band(low, self.NZ)

    def set_spectral_state(self, om2, fnm1=None, uc_low=None):
        """Load om2/fnm1 (and optionally the velocity low band) from host arrays."""
        self._field.set_state(om2, fnm1, uc_low)

    def flow_eddy_metrics(self):
        """(U, L, tau_L) as turbo_simulator.py:764-810 computes them."""
        d = self._field.diagnostics()
        return d["U"], d["L"], d["tau_l"]

    def diagnostics(self) -> dict:
        return self._field.diagnostics()


def create_dns_state(N: int = 8, Re: float = 1e5, K0: float = 100.0, CFL: float = 0.75,
                     backend: str = "gb300", seed: int = 1, skip_pao: bool = False,
                     populate_compact_ur: bool = True, start_spectrum: SPECTRUM = "KM3",
                     precision: str = "fp32", generator: str = "host") -> DnsState:
    """Allocate the GB300 state and run the PAO/KM3 generator (turbo_simulator.py:878-1054).

    `generator="host"` (default): the reference's own initial field bit for bit
    (C++ LCG and shell sums, NumPy float32 cos/sin/exp as the reference evaluates
    them; `_lib.pao_generate`), then uploaded.  `"device"`: pal_generate, the
    per-mode work on the GPU (N=4096 in ~0.04 s), whose CUDA float32 functions
    differ from NumPy's by a few ulp (<= 4e-7 relative)."""
    if backend not in ("gb300", "gpu", "auto"):
        raise ValueError(f"backend {backend!r}: this module is the GB300 backend (no CPU path)")
    S = DnsState(N, Re, K0, CFL, seed, start_spectrum, precision, populate_compact_ur)
    if skip_pao:
        return S
    if generator == "device":
        uc, st = S.field.generate(K0, Re, seed, start_spectrum)
    elif generator == "host":
        om2, uc, st = L.pao_generate(N, K0, Re, seed, start_spectrum)
    else:
        raise ValueError(f"generator {generator!r}: 'device' or 'host'")
    print(f"--- INITIALIZING GB300 --- N={N}, K0={int(K0)}, Re={float(Re):,.1f}, {start_spectrum}")
    print(f" Energy      = {st['Energy']:.8g}")
    print(f" WiWi        = {st['WiWi']:.8g}")
    print(f" Viscosity   = {st['visc']:.8g}")
    print(f" PAO seed in = {seed}")
    print(f" PAO seed out= {st['seed_out']}")
    if generator == "host":
        S.set_spectral_state(om2, None, uc)
    S.uc_init = np.asarray(uc, np.complex64)
    S.visc = float(st["visc"])
    S.dt, S.cn, S.cnm1 = 0.0, 1.0, 0.0
    return S


VAR_U, VAR_V, VAR_ENERGY, VAR_OMEGA, VAR_STREAM = 0, 1, 2, 3, 4


def dns_kinetic(S: DnsState) -> None:
    """|u| = sqrt(u^2 + v^2) on the 3/2 grid into ur_full[2] (turbo_simulator.py:2629-2636)."""
    S.field.vis(VAR_ENERGY, out=S.ur_full.plane2())


def dns_om2_phys(S: DnsState) -> None:
    """Physical vorticity from om2 into ur_full[2] (turbo_simulator.py:2684-2687)."""
    S.field.vis(VAR_OMEGA, out=S.ur_full.plane2())


def dns_stream_func(S: DnsState) -> None:
    """Streamfunction om2/(K2 + 1e-30) on the 3/2 grid into ur_full[2] (turbo_simulator.py:2690-2708)."""
    S.field.vis(VAR_STREAM, out=S.ur_full.plane2())


def frame_pixels(S: DnsState, var: int = VAR_U):
    """uint8 display frame of DnsSimulator's variable selector (turbo_wrapper.py:353-413)."""
    return S.field.vis(var, field=False, pixels=True)[1]


def dns_step2a(S: DnsState) -> None:
    S.field.step2a()


def dns_step2b(S: DnsState) -> None:
    S.field.step2b()


def dns_step3(S: DnsState, fuse: bool = True) -> None:
    S.field.step3()
    object.__setattr__(S, "cnm1", float(S.cn))


def dns_step_ls_imex_rk3(S: DnsState) -> None:
    S.field.step_rk3()


def compute_cflm(S: DnsState) -> float:
    return S.field.compute_cflm()


def sync_time_scalars_from_device(S: DnsState) -> None:
    sc = S.field.scalars()
    for k in ("dt", "cn", "cnm1"):
        object.__setattr__(S, k, sc[k])


def next_dt(S: DnsState, sync_host: bool = False):
    """NEXTDT on the device; with sync_host the host mirrors are refreshed and CFLM returned."""
    cflm = S.field.next_dt(sync_host)
    if sync_host:
        sync_time_scalars_from_device(S)
        return cflm
    return None


def _init_dt(S: DnsState) -> float:
    dns_step2a(S)
    cflm0 = compute_cflm(S)
    S.dt = S.cflnum / (cflm0 * math.pi)
    S.cn = 1.0
    S.cnm1 = 0.0
    S.t = 0.0
    return cflm0


def run_dns(N: int = 8, Re: float = 100, K0: float = 10.0, STEPS: int = 2, CFL: float = 0.75,
            backend: str = "gb300", start_spectrum: SPECTRUM = "KM3", UPDATE: int = 100,
            method: TimeStepper = "CNAB2", precision: str = "fp32"):
    """The sim CLI driver (turbo_simulator.py:2744-2858) on the GB300 kernels."""
    if method == "CHECK":
        compare_time_steppers(N, Re, K0, STEPS, CFL, backend, start_spectrum, UPDATE, precision)
        return None
    if method not in _METHODS:
        raise ValueError(f"unknown time stepper: {method}")
    print("--- RUN DNS (GB300) ---")
    print(f" N = {N}  Re = {Re}  K0 = {K0}  Steps = {STEPS}  CFL = {CFL}  Update = {UPDATE}  "
          f"Spectrum = {start_spectrum}  Method = {method}  precision = {precision}")
    seed = pao_seed_from_env(1)
    S = create_dns_state(N=N, Re=Re, K0=K0, CFL=CFL, backend=backend, seed=seed,
                         start_spectrum=start_spectrum, populate_compact_ur=False, precision=precision)
    cflm0 = _init_dt(S)
    print(f" [NEXTDT INIT] CFLM={cflm0:11.4f} DT={S.dt:11.7f} CN={S.cn:11.7f}")
    f = S.field
    f.set_scalar("it", 0)
    f.set_scalar("t", 0.0)
    S.sync()
    t0 = time.perf_counter()
    marks = sorted({1, STEPS} | set(range(UPDATE, STEPS + 1, UPDATE))) if UPDATE > 0 else [STEPS]
    done = 0
    for m in marks:
        f.step(method, m - done, update=0, final_update=False)
        done = m
        before = f.scalars()  # t already includes this step's dt_old
        cflm = next_dt(S, sync_host=True)
        S.t, S.it = before["t"], before["it"]
        _, _, tau_l = S.flow_eddy_metrics()
        print(f" ITERATION {m:6d} T={before['t'] - before['dt']:12.10f} DT={S.dt:10.8f} "
              f"CN={S.cn:10.8f} CFLM={cflm:.6f} TAU_L={tau_l:.6f}")
    S.sync()
    elap = time.perf_counter() - t0
    fps = STEPS / elap if elap > 0 else 0.0
    print(f" Elapsed time for {STEPS} steps (s) = {elap:.8g}")
    print(f" Final T={S.t:.8g}  CN={S.cn:.8g}  DT={S.dt:.8g}")
    print(f" FPS = {fps:.8g}")
    return S


def compare_time_steppers(N, Re, K0, STEPS, CFL, backend, start_spectrum, UPDATE, precision="fp32"):
    """CHECK mode: CNAB2 vs LS-IMEX-RK3 from the same seed (turbo_simulator.py:2877-2903)."""
    a = run_dns(N, Re, K0, STEPS, CFL, backend, start_spectrum, UPDATE, "CNAB2", precision)
    b = run_dns(N, Re, K0, STEPS, CFL, backend, start_spectrum, UPDATE, "LS_IMEX_RK3", precision)
    oa, ob = a.om2.astype(np.complex128), b.om2.astype(np.complex128)
    l2 = float(np.linalg.norm(ob - oa) / max(np.linalg.norm(oa), 1e-30))
    linf = float(np.abs(ob - oa).max() / max(np.abs(oa).max(), 1e-30))
    print("--- CHECK RESULT ---")
    print(f" OM2 relative L2={l2:.6e} Linf={linf:.6e}")
    return l2, linf


def main():
    args = sys.argv[1:]
    N = int(args[0]) if len(args) > 0 else 512
    Re = float(args[1]) if len(args) > 1 else 10000
    K0 = float(args[2]) if len(args) > 2 else 10.0
    STEPS = int(args[3]) if len(args) > 3 else 1001
    CFL = float(args[4]) if len(args) > 4 else 0.25
    UPDATE = int(float(args[6])) if len(args) > 6 else 100
    SPEC = args[7].upper() if len(args) > 7 else "KM3"
    METHOD = args[8].upper() if len(args) > 8 else "CNAB2"
    PREC = args[9].lower() if len(args) > 9 else "fp32"
    run_dns(N=N, Re=Re, K0=K0, STEPS=STEPS, CFL=CFL, start_spectrum=SPEC, UPDATE=UPDATE, method=METHOD,
            precision=PREC)


if __name__ == "__main__":
    main()


class Ensemble:
    """Many independent fields (members) of possibly different N, stepped together.

    Each member keeps its own viscosity, CFL target and adaptive dt.  One kernel
    launch per group of equal N per pass; with ``graph=True`` the launch
    sequence of a step call is captured once as a CUDA graph and replayed.
    """

    def __init__(self, Ns, precision="fp32", Re=1e4, cfl=0.5):
        self.lib = L.load()
        self.Ns = [int(n) for n in Ns]
        self.precision = precision
        self.cdt = np.complex64 if precision == "fp32" else np.complex128
        arr = (L._I * len(self.Ns))(*self.Ns)
        h = L._H()
        rc = self.lib.pal_ensemble_create(len(self.Ns), arr, _PREC[precision], float(Re), float(cfl), h)
        if rc != L.PAL_OK:
            raise L.PalError(rc, self._err(None))
        self.h = h

    def _err(self, h):
        buf = L.ctypes.create_string_buffer(512)
        self.lib.pal_ensemble_last_error(h, buf, len(buf))
        return buf.value.decode()

    def _ck(self, rc):
        if rc != L.PAL_OK:
            raise (ValueError(self._err(self.h)) if rc == L.PAL_ERR_INVALID else L.PalError(rc, self._err(self.h)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.pal_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def autotune(self):
        """Re-tune each size group on its batched shape (before any member is set)."""
        self._ck(self.lib.pal_ensemble_autotune(self.h))

    def variant(self, N: int) -> str:
        buf = L.ctypes.create_string_buffer(256)
        self._ck(self.lib.pal_ensemble_get_variant(self.h, int(N), buf, len(buf)))
        return buf.value.decode()

    def set_member(self, m, om2, fnm1=None, uc_low=None):
        om2 = np.ascontiguousarray(om2, dtype=self.cdt)
        f = None if fnm1 is None else np.ascontiguousarray(fnm1, dtype=self.cdt)
        u = None if uc_low is None else np.ascontiguousarray(uc_low, dtype=self.cdt)
        self._ck(self.lib.pal_ensemble_set_member(self.h, int(m), L.ptr(om2), None if f is None else L.ptr(f),
                                                  None if u is None else L.ptr(u)))

    def set_scalar(self, m, which, value):
        idx = {"t": L.PAL_SC_T, "dt": L.PAL_SC_DT, "cn": L.PAL_SC_CN, "cnm1": L.PAL_SC_CNM1,
               "visc": L.PAL_SC_VISC, "cflnum": L.PAL_SC_CFLNUM}[which]
        self._ck(self.lib.pal_ensemble_set_scalar(self.h, int(m), idx, float(value)))

    def init_dt(self):
        self._ck(self.lib.pal_ensemble_init_dt(self.h))

    def step(self, method="CNAB2", nsteps=1, update=1, graph=True):
        self._ck(self.lib.pal_ensemble_step(self.h, _METHODS[method], int(nsteps), int(update), int(bool(graph))))

    def om2(self, m):
        a = np.empty((self.Ns[m], self.Ns[m] // 2), self.cdt)
        self._ck(self.lib.pal_ensemble_get_member(self.h, int(m), L.PAL_FIELD_OM2, L.ptr(a)))
        return a

    def fnm1(self, m):
        a = np.empty((self.Ns[m], self.Ns[m] // 2), self.cdt)
        self._ck(self.lib.pal_ensemble_get_member(self.h, int(m), L.PAL_FIELD_FNM1, L.ptr(a)))
        return a

    def scalars(self, m):
        v = [L._D() for _ in range(4)]
        it = L.ctypes.c_longlong()
        self._ck(self.lib.pal_ensemble_get_scalars(self.h, int(m), *[L.ctypes.byref(x) for x in v],
                                                   L.ctypes.byref(it)))
        return dict(zip(("t", "dt", "cn", "cflm"), [x.value for x in v]), it=it.value)

    def stream_ptr(self):
        p = L._P()
        self._ck(self.lib.pal_ensemble_get_stream(self.h, L.ctypes.byref(p)))
        return p.value

    def synchronize(self):
        self._ck(self.lib.pal_ensemble_synchronize(self.h))


# Spectrum API of the reference module (turbo_simulator.py:2225-2622).
from .spectrum import (  # noqa: E402,F401
    SpectrumAverageState,
    SpectrumSample,
    compute_energy_spectrum_uv_bins,
    initialize_spectrum_average_from_sample,
    mark_spectrum_average_since_restart,
    sample_and_update_spectrum_average,
    save_energy_spectrum_csv_data,
    save_energy_spectrum_uv_csv,
    save_spectrum_average_csv,
    spectrum_average_kind,
    spectrum_average_mean_energy,
    update_spectrum_average,
)
