"""NetCDF restart files: the reference's `restart.nc` layout, written and read
on the host around the GB300 state.

Mirrors the restart helpers of the reference GUI (palinstrophy/turbo_main.py):
  _complex_array_to_host     1278-1281
  _restart_dims              1283-1291
  _write_complex_netcdf      1293-1304
  _read_complex_netcdf       1306-1310
  _dump_restart_netcdf       1312-1338  -> dump_restart_netcdf(S, folder)
  _load_restart_netcdf       1373-1503  -> load_restart_netcdf(folder) (state part only)
and the file description in README.md:275-301.

Same variable names, dimension names, shapes and attribute names:
  uc_real/uc_imag     (uc_z, uc_k, uc_component) = (N, 3N/4+1, 3)  float32
  om2_real/om2_imag   (om2_z, om2_x_half)        = (N, N/2)        float32
  fnm1_real/fnm1_imag (fnm1_z, fnm1_x_half)      = (N, N/2)        float32
  attributes format_version, Nbase, Re, K0, start_spectrum, visc, cflnum,
  seed_init, t, dt, cn, cnm1, it.

Container: the reference writes NETCDF4 (an HDF5 file, zlib level 4 with
shuffle) through the netCDF4 package.  Neither netCDF4 nor an HDF5 library is
a dependency of this package, so files are written in the netCDF classic 64-bit-offset
format (CDF-2) with scipy.io.netcdf_file: the netCDF library opens classic and
NETCDF4 files through the same Dataset call, so the reference's loader reads
these files unchanged.  Reading a NETCDF4/HDF5 file written by the reference
needs the netCDF4 package; without it the loader raises a RuntimeError saying
so.  Integers are stored as 32-bit (classic has no 64-bit integer attribute);
floats as 64-bit doubles, as the reference stores Python floats.

Stale-velocity quirk of the reference: `S.uc` is filled once by the initial
generator (turbo_simulator.py:1221) and never updated by stepping, so the
saved `uc` is the initial velocity; on load `uc_full` is rebuilt from it
(turbo_main.py:1443-1445) and step2a turns that stale spectrum into the
physical velocity used by the first step after the load, while om2 and fnm1
are current.  `stale_uc=True` (default) reproduces this on both sides;
`stale_uc=False` saves the velocity of the current om2 and, on load, rebuilds
the velocity from om2 (the inversion of turbo_simulator.py:1555-1585), so a
loaded run continues exactly where the saved one stopped.
"""
from __future__ import annotations

import os
import time

import numpy as np

RESTART_FILE = "restart.nc"
FORMAT_VERSION = 1


def _complex_array_to_host(arr) -> np.ndarray:
    host = arr.get() if hasattr(arr, "get") else np.asarray(arr)
    return np.asarray(host)


def _restart_dims(name: str, shape: tuple[int, ...]) -> tuple[str, ...]:
    if name == "uc":
        return ("uc_z", "uc_k", "uc_component")
    if name == "om2":
        return ("om2_z", "om2_x_half")
    if name == "fnm1":
        return ("fnm1_z", "fnm1_x_half")
    return tuple(f"{name}_dim_{i}" for i in range(len(shape)))


def _write_complex_netcdf(ds, name: str, arr) -> None:
    host = _complex_array_to_host(arr)
    dims = _restart_dims(name, host.shape)
    for dim, size in zip(dims, host.shape):
        ds.createDimension(dim, int(size))
    real = ds.createVariable(f"{name}_real", "f4", dims)
    imag = ds.createVariable(f"{name}_imag", "f4", dims)
    real[:] = np.asarray(host.real, dtype=np.float32)
    imag[:] = np.asarray(host.imag, dtype=np.float32)


def _read_complex_netcdf(ds, name: str) -> np.ndarray:
    real = np.asarray(ds.variables[f"{name}_real"][:], dtype=np.float32)
    imag = np.asarray(ds.variables[f"{name}_imag"][:], dtype=np.float32)
    return (real + 1j * imag).astype(np.complex64, copy=False)


def _attr(ds, name):
    v = ds._attributes[name] if hasattr(ds, "_attributes") else ds.getncattr(name)
    if isinstance(v, bytes):
        return v.decode()
    if isinstance(v, np.ndarray) and v.size == 1:
        return v.reshape(()).item()
    return v.item() if hasattr(v, "item") else v


def _open_for_read(path):
    with open(path, "rb") as f:
        magic = f.read(4)
    if magic[:3] == b"CDF":
        from scipy.io import netcdf_file
        return netcdf_file(path, "r", mmap=False)
    if magic == b"\x89HDF":
        try:
            from netCDF4 import Dataset  # the reference's own reader, if installed
        except ImportError as e:
            raise RuntimeError(f"{path} is a NETCDF4/HDF5 file; reading it needs the netCDF4 package, "
                               "which is not installed") from e
        ds = Dataset(path, "r")
        ds.set_auto_mask(False)
        return ds
    raise RuntimeError(f"{path} is not a netCDF file (magic {magic!r})")


# -- velocity spectra in the reference's compact `uc` layout -------------------

def uc_from_low_band(uc_low: np.ndarray, N: int) -> np.ndarray:
    """(2, N, N/2) low-band velocity -> reference `uc` (N, 3N/4+1, 3), components 0, 1
    at x < N/2 (turbo_simulator.py:1193-1198, 1221); the rest is zero."""
    uc = np.zeros((N, 3 * N // 4 + 1, 3), np.complex64)
    uc[:, : N // 2, 0] = uc_low[0]
    uc[:, : N // 2, 1] = uc_low[1]
    return uc


def low_band_from_uc(uc: np.ndarray, N: int) -> np.ndarray:
    """Reference `uc` -> (2, N, N/2): the part that survives step2a's de-aliasing
    (columns kx >= N/2 are zeroed, turbo_simulator.py:2020-2026)."""
    if uc.shape != (N, 3 * N // 4 + 1, 3):
        raise ValueError(f"uc has shape {uc.shape}, expected {(N, 3 * N // 4 + 1, 3)}")
    return np.ascontiguousarray(np.stack([uc[:, : N // 2, 0], uc[:, : N // 2, 1]]), dtype=np.complex64)


def velocity_from_om2(om2: np.ndarray) -> np.ndarray:
    """(u^, v^) of om2 as turbo_simulator.py:1555-1585 forms them (FP32):
    u^ = -i gamma om2 / K^2, v^ = i alpha om2 / K^2 for kx >= 1;
    u^ = -i om2 / gamma (0 at gamma = 0), v^ = 0 on the kx = 0 column."""
    N = om2.shape[0]
    nh = N // 2
    om = om2.astype(np.complex64)
    kz = np.arange(N)
    gamma = np.where(kz < nh, kz, kz - N).astype(np.float32)
    alfa = np.arange(nh, dtype=np.float32)
    out = np.zeros((2, N, nh), np.complex64)
    if nh > 1:
        K2 = alfa[None, 1:] ** 2 + gamma[:, None] ** 2
        invK2 = (np.float32(1.0) / K2).astype(np.float32)
        out[0, :, 1:] = (om[:, 1:] * invK2 * gamma[:, None]) * np.complex64(-1j)
        out[1, :, 1:] = (om[:, 1:] * invK2 * alfa[None, 1:]) * np.complex64(1j)
    with np.errstate(divide="ignore"):
        inv_g0 = np.where(gamma != 0, np.float32(1.0) / np.where(gamma != 0, gamma, 1), 0).astype(np.float32)
    out[0, :, 0] = np.complex64(-1j) * om[:, 0] * inv_g0
    return out


# -- dump / load ---------------------------------------------------------------

ATTRS = ("format_version", "Nbase", "Re", "K0", "start_spectrum", "visc", "cflnum", "seed_init",
         "t", "dt", "cn", "cnm1", "it")
_INT_ATTRS = {"format_version", "Nbase", "seed_init", "it"}


def write_restart_file(path: str, attrs: dict, uc, om2, fnm1) -> str:
    """Write one restart file: the attributes (ATTRS, in that order) and the three
    complex fields as float32 real/imag variables (turbo_main.py:1319-1336)."""
    from scipy.io import netcdf_file

    ds = netcdf_file(path, "w", version=2)
    try:
        for name in ATTRS:
            v = attrs[name]
            if name == "start_spectrum":
                setattr(ds, name, str(v))
            elif name in _INT_ATTRS:
                setattr(ds, name, np.int32(v))
            else:
                setattr(ds, name, np.float64(v))
        _write_complex_netcdf(ds, "uc", uc)
        _write_complex_netcdf(ds, "om2", om2)
        _write_complex_netcdf(ds, "fnm1", fnm1)
    finally:
        ds.close()
    return path


def dump_restart_netcdf(S, folder_path: str, stale_uc: bool = True) -> str:
    """Write `restart.nc` for a GB300 DnsState into folder_path (turbo_main.py:1312-1338)."""
    from . import turbo_simulator as ts

    ts.sync_time_scalars_from_device(S)
    sc = S.field.scalars()
    N = int(S.Nbase)
    om2 = S.om2
    if stale_uc:
        uc_low = S.uc_init if getattr(S, "uc_init", None) is not None else np.zeros((2, N, N // 2), np.complex64)
    else:
        uc_low = velocity_from_om2(om2)
    os.makedirs(folder_path, exist_ok=True)
    attrs = {"format_version": FORMAT_VERSION, "Nbase": N, "Re": S.Re, "K0": S.K0,
             "start_spectrum": S.start_spectrum, "visc": sc["visc"], "cflnum": sc["cflnum"],
             "seed_init": S.seed_init, "t": sc["t"], "dt": sc["dt"], "cn": sc["cn"], "cnm1": sc["cnm1"],
             "it": sc["it"]}
    path = write_restart_file(os.path.join(folder_path, RESTART_FILE), attrs, uc_from_low_band(uc_low, N),
                              om2, S.fnm1)
    print(f"[SAVE] NetCDF restart written to {path}")
    return path


def read_restart_netcdf(folder_path: str) -> dict:
    """Attributes and arrays of a restart file, as the reference's loader reads them
    (turbo_main.py:1382-1400)."""
    path = os.path.join(folder_path, RESTART_FILE)
    if not os.path.isfile(path):
        raise FileNotFoundError(f"No {RESTART_FILE} in {folder_path}")
    ds = _open_for_read(path)
    try:
        out = {
            "Nbase": int(_attr(ds, "Nbase")),
            "Re": float(_attr(ds, "Re")),
            "K0": float(_attr(ds, "K0")),
            "start_spectrum": str(_attr(ds, "start_spectrum")),
            "visc": float(_attr(ds, "visc")),
            "cflnum": float(_attr(ds, "cflnum")),
            "seed_init": int(_attr(ds, "seed_init")),
            "t": float(_attr(ds, "t")),
            "dt": float(_attr(ds, "dt")),
            "cn": float(_attr(ds, "cn")),
            "cnm1": float(_attr(ds, "cnm1")),
            "it": int(_attr(ds, "it")),
            "uc": _read_complex_netcdf(ds, "uc"),
            "om2": _read_complex_netcdf(ds, "om2"),
            "fnm1": _read_complex_netcdf(ds, "fnm1"),
        }
    finally:
        ds.close()
    N = out["Nbase"]
    for k in ("om2", "fnm1"):
        if out[k].shape != (N, N // 2):
            raise ValueError(f"{k} has shape {out[k].shape}, expected {(N, N // 2)}")
    return out


def load_restart_netcdf(folder_path: str, precision: str = "fp32", stale_uc: bool = True):
    """Recreate a GB300 DnsState from `restart.nc` (turbo_main.py:1373-1445): same N,
    Re, K0, spectrum, CFL and seed, om2 / fnm1 / scalars restored, then step2a."""
    from . import turbo_simulator as ts

    t0 = time.time()
    d = read_restart_netcdf(folder_path)
    N = d["Nbase"]
    S = ts.create_dns_state(N, d["Re"], d["K0"], d["cflnum"], seed=d["seed_init"], skip_pao=True,
                            start_spectrum=d["start_spectrum"], precision=precision)
    uc_low = low_band_from_uc(d["uc"], N)
    S.uc_init = uc_low
    S.set_spectral_state(d["om2"], d["fnm1"], uc_low if stale_uc else None)
    S.visc = d["visc"]
    S.cflnum = d["cflnum"]
    S.dt, S.cn, S.cnm1 = d["dt"], d["cn"], d["cnm1"]
    S.t, S.it = d["t"], d["it"]
    S.field.set_scalar("t", d["t"])
    S.field.set_scalar("it", d["it"])
    ts.dns_step2a(S)
    print(f"[LOAD] Restored case from {folder_path}: N={N}, Re={d['Re']:.4e}, K0={d['K0']}, "
          f"spectrum={d['start_spectrum']}, t={d['t']:.6e}, it={d['it']} ({time.time() - t0:.2f}s)")
    return S
