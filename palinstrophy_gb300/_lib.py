"""ctypes binding of libpalgpu.so (the C ABI declared in include/palgpu.h).

The library is built in-tree by ``palinstrophy_gb300.build``.  There is no
fallback: if the library is missing or the GPU call fails, the caller gets an
exception.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpalgpu.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "palgpu.h")

PAL_OK = 0
PAL_ERR_INVALID = -1
PAL_ERR_CUDA = -2
PAL_ERR_OOM = -3
PAL_ERR_STATE = -4
PAL_ERR_NONFINITE = -5
PAL_ERR_TIMEOUT = -6
PAL_DBG_SKIP_FIRST_WAIT = 0
PAL_FP32, PAL_FP64 = 0, 1
PAL_CNAB2, PAL_LS_IMEX_RK3 = 0, 1
PAL_FIELD_OM2, PAL_FIELD_FNM1, PAL_FIELD_UR_U, PAL_FIELD_UR_V = 0, 1, 2, 3
PAL_SPEC_KM3, PAL_SPEC_PAO = 0, 1
PAL_SC_T, PAL_SC_DT, PAL_SC_CN, PAL_SC_CNM1, PAL_SC_VISC, PAL_SC_CFLNUM, PAL_SC_IT = range(7)


class PalDiag(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "U", "L", "tau_l", "E", "Z", "P", "kmax2", "pal_over_ens_kmax2", "cflm", "energy_joules")] + [
        ("nonfinite", ctypes.c_int)]


class PalError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libpalgpu error {code}: {msg}")
        self.code = code


_H = ctypes.c_void_p
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_DP = ctypes.POINTER(ctypes.c_double)
_SIGS = {
    "pal_create": (_I, [_I, _I, _D, _D, ctypes.POINTER(_H)]),
    "pal_destroy": (_I, [_H]),
    "pal_supported": (_I, [_I, _I]),
    "pal_generate": (_I, [_H, _D, _D, _I, _I, _P, ctypes.POINTER(_D), ctypes.POINTER(_I)]),
    "pal_ensemble_autotune": (_I, [_H]),
    "pal_ensemble_get_variant": (_I, [_H, _I, ctypes.c_char_p, ctypes.c_size_t]),
    "pal_device_info": (_I, [ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.c_char_p, ctypes.c_size_t]),
    "pal_set_spectral_state": (_I, [_H, _P, _P]),
    "pal_set_velocity_spectrum": (_I, [_H, _P]),
    "pal_set_scalars": (_I, [_H, _D, _D, _D, _D, _D, _D, ctypes.c_longlong]),
    "pal_get_scalars": (_I, [_H, _DP, _DP, _DP, _DP, _DP, _DP, ctypes.POINTER(ctypes.c_longlong)]),
    "pal_set_scalar": (_I, [_H, _I, _D]),
    "pal_step2a": (_I, [_H]),
    "pal_step2b": (_I, [_H]),
    "pal_step3": (_I, [_H]),
    "pal_step_rk3": (_I, [_H]),
    "pal_step": (_I, [_H, _I, _I, _I, _I]),
    "pal_compute_cflm": (_I, [_H, _DP]),
    "pal_next_dt": (_I, [_H, _I, _DP]),
    "pal_diagnostics": (_I, [_H, ctypes.POINTER(PalDiag)]),
    "pal_get_field": (_I, [_H, _I, _P]),
    "pal_adjoint_palinstrophy": (_I, [_H, _I, _I, _DP, _P]),
    "pal_vis_field": (_I, [_H, _I, _P, ctypes.POINTER(ctypes.c_ubyte)]),
    "pal_energy_spectrum": (_I, [_H, _I, _D, _D, _DP, ctypes.POINTER(_I)]),
    "pal_field_device_ptr": (_I, [_H, _I, ctypes.POINTER(_P)]),
    "pal_materialize_physical": (_I, [_H]),
    "pal_synchronize": (_I, [_H]),
    "pal_get_stream": (_I, [_H, ctypes.POINTER(_P)]),
    "pal_set_debug": (_I, [_H, _I, _I]),
    "pal_fp64_peak": (_I, [_DP, _DP]),
    "pal_get_variant": (_I, [_H, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                             ctypes.c_char_p, ctypes.c_size_t]),
    "pal_set_variant": (_I, [_H, _I, _I]),
    "pal_get_occupancy": (_I, [_H, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "pal_profile_kernels": (_I, [_H, _I, _I, _DP, _DP, ctypes.POINTER(_I)]),
    "pal_last_error": (_I, [_H, ctypes.c_char_p, ctypes.c_size_t]),
    "pal_ensemble_create": (_I, [_I, ctypes.POINTER(_I), _I, _D, _D, ctypes.POINTER(_H)]),
    "pal_ensemble_destroy": (_I, [_H]),
    "pal_ensemble_set_member": (_I, [_H, _I, _P, _P, _P]),
    "pal_ensemble_set_scalar": (_I, [_H, _I, _I, _D]),
    "pal_ensemble_init_dt": (_I, [_H]),
    "pal_ensemble_step": (_I, [_H, _I, _I, _I, _I]),
    "pal_ensemble_get_member": (_I, [_H, _I, _I, _P]),
    "pal_ensemble_get_scalars": (_I, [_H, _I, _DP, _DP, _DP, _DP, ctypes.POINTER(ctypes.c_longlong)]),
    "pal_ensemble_get_stream": (_I, [_H, ctypes.POINTER(_P)]),
    "pal_ensemble_synchronize": (_I, [_H]),
    "pal_ensemble_last_error": (_I, [_H, ctypes.c_char_p, ctypes.c_size_t]),
    "pal_step_noalloc": (_I, [_I, _I, _I, _D, _D, _D, _D, _P, _P, _P]),
    "pal_pao_generate": (_I, [_I, _D, _D, _I, _I, _P, _P, _DP, ctypes.POINTER(_I)]),
    "pal_pao_draws": (_I, [_I, _I, _P, ctypes.POINTER(_I)]),
    "pal_pao_build": (_I, [_I, _D, _D, _I, _I, _P, _P, _P, _P, _P, _DP]),
}

_lib = None


def header_symbols():
    """Names of every entry point declared in include/palgpu.h."""
    with open(HEADER_PATH) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*int\s+(pal_\w+)\s*\(", text, flags=re.M)))


def load():
    """Load libpalgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing; build it with `python -m palinstrophy_gb300.build`")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error(h=None) -> str:
    buf = ctypes.create_string_buffer(1024)
    load().pal_last_error(h, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, h=None):
    if rc != PAL_OK:
        msg = last_error(h)
        if rc in (PAL_ERR_INVALID,):
            raise ValueError(msg)
        raise PalError(rc, msg)
    return rc


def supported(N, precision="fp32") -> bool:
    """True if kernels for this grid size and precision are compiled in."""
    prec = {"fp32": PAL_FP32, "fp64": PAL_FP64}[precision]
    return load().pal_supported(int(N), prec) == 1


def ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def pao_generate(N, K0, Re, seed, spectrum="KM3"):
    """Host generator: returns (om2 (N,N/2) c64, uc_low (2,N,N/2) c64, stats dict).

    The reference's own field, bit for bit on the machine it runs on: the serial
    LCG draws (pal_pao_draws) and everything after the three per-mode float32
    transcendental values (pal_pao_build) run in C++; those three values --
    cos and sin of the phase 2 pi v and exp(-(k/K0)^2) -- are NumPy's float32
    ufuncs, as the reference evaluates them (turbo_simulator.py:287-318).
    """
    N = int(N)
    if N < 8 or N % 4:
        raise ValueError("N must be a multiple of 4 and >= 8")
    spec = {"KM3": PAL_SPEC_KM3, "PAO": PAL_SPEC_PAO}[spectrum.upper()]
    lib = load()
    nh = N // 2
    v = np.empty((N, nh), np.float32)
    so = ctypes.c_int(0)
    check(lib.pal_pao_draws(N, int(seed), ptr(v), ctypes.byref(so)))
    pi = np.float32(3.14159265358979)
    th = (np.float32(2.0) * pi) * v
    cos_th = np.cos(th)
    sin_th = np.sin(th)
    alfa = np.arange(nh, dtype=np.float32)
    z = np.arange(N)
    gamma = np.where(z < nh, z, z - N).astype(np.float32)
    k2 = (gamma * gamma)[:, None] + (alfa * alfa)[None, :]
    k = np.sqrt(k2)
    t = k / np.float32(K0)
    exp_g = np.exp((-t) * t)
    om2 = np.zeros((N, nh), np.complex64)
    uc = np.zeros((2, N, nh), np.complex64)
    st = (ctypes.c_double * 3)()
    check(lib.pal_pao_build(N, float(K0), float(Re), int(seed), spec, ptr(cos_th), ptr(sin_th), ptr(exp_g),
                            ptr(om2), ptr(uc), st))
    # om2 = i (gamma u1 - alfa u3) with NumPy's complex64 arithmetic, so that even
    # the signs of zero modes are the reference's (turbo_simulator.py:1314-1361)
    d = gamma[:, None] * uc[0] - alfa[None, :] * uc[1]
    om2 = np.asarray(-d.imag + 1j * d.real, dtype=np.complex64)
    return om2, uc, {"Energy": st[0], "WiWi": st[1], "visc": st[2], "seed_out": so.value}


def pao_generate_libm(N, K0, Re, seed, spectrum="KM3"):
    """The same generator with the C library's float32 cos/sin/exp (pal_pao_generate)."""
    spec = {"KM3": PAL_SPEC_KM3, "PAO": PAL_SPEC_PAO}[spectrum.upper()]
    om2 = np.zeros((N, N // 2), np.complex64)
    uc = np.zeros((2, N, N // 2), np.complex64)
    st = (ctypes.c_double * 3)()
    so = ctypes.c_int(0)
    check(load().pal_pao_generate(int(N), float(K0), float(Re), int(seed), spec, ptr(om2), ptr(uc), st,
                                  ctypes.byref(so)))
    return om2, uc, {"Energy": st[0], "WiWi": st[1], "visc": st[2], "seed_out": so.value}


def fp64_peak():
    """(TFLOP/s, ms) of the FP64 FMA microbenchmark on the current GPU (pal_fp64_peak)."""
    tf, ms = ctypes.c_double(), ctypes.c_double()
    check(load().pal_fp64_peak(ctypes.byref(tf), ctypes.byref(ms)))
    return tf.value, ms.value
