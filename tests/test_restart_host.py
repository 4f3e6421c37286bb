"""Restart file layout and host logic (no GPU): the reference's restart.nc
variables, dimensions and attributes (turbo_main.py:1283-1338), the read path
(turbo_main.py:1382-1400), the compact `uc` layout and the om2 -> velocity
inversion used by the non-stale save."""

import numpy as np
import pytest

from oracle import dns_oracle as do
from palinstrophy_gb300 import restart as rs


def _attrs(N):
    return {"format_version": 1, "Nbase": N, "Re": 1.0e4 / 3.0, "K0": 10.0, "start_spectrum": "KM3",
            "visc": float(np.float32(3e-4)), "cflnum": 0.75, "seed_init": 4895, "t": 0.123456789012345,
            "dt": 1.0e-3 / 7.0, "cn": 0.987654321, "cnm1": 1.0123456789, "it": 1234}


def _fields(N, seed=0):
    rng = np.random.default_rng(seed)
    c = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    return c(N, 3 * N // 4 + 1, 3), c(N, N // 2), c(N, N // 2)


def test_file_has_reference_layout(tmp_path):
    from scipy.io import netcdf_file
    N = 16
    uc, om2, fnm1 = _fields(N)
    path = rs.write_restart_file(str(tmp_path / rs.RESTART_FILE), _attrs(N), uc, om2, fnm1)
    with open(path, "rb") as f:
        assert f.read(4) == b"CDF\x02"  # classic, 64-bit offsets
    ds = netcdf_file(path, "r", mmap=False)
    try:
        assert set(ds._attributes) == set(rs.ATTRS)
        assert ds._attributes["start_spectrum"] == b"KM3"
        for k in ("format_version", "Nbase", "seed_init", "it"):
            assert ds._attributes[k].dtype == np.int32
        for k in ("Re", "K0", "visc", "cflnum", "t", "dt", "cn", "cnm1"):
            assert ds._attributes[k].dtype == np.float64
        want = {"uc": ("uc_z", "uc_k", "uc_component"), "om2": ("om2_z", "om2_x_half"),
                "fnm1": ("fnm1_z", "fnm1_x_half")}
        assert set(ds.variables) == {f"{n}_{p}" for n in want for p in ("real", "imag")}
        for n, dims in want.items():
            for p in ("real", "imag"):
                v = ds.variables[f"{n}_{p}"]
                assert v.dimensions == dims
                assert v.data.dtype.kind == "f" and v.data.dtype.itemsize == 4
        assert ds.variables["uc_real"].data.shape == (N, 3 * N // 4 + 1, 3)
        assert ds.variables["om2_imag"].data.shape == (N, N // 2)
    finally:
        ds.close()


def test_round_trip_is_exact(tmp_path):
    N = 32
    uc, om2, fnm1 = _fields(N, 1)
    a = _attrs(N)
    rs.write_restart_file(str(tmp_path / rs.RESTART_FILE), a, uc, om2, fnm1)
    d = rs.read_restart_netcdf(str(tmp_path))
    for k, v in a.items():
        if k == "format_version":
            continue
        assert d[k] == v, k
    assert np.array_equal(d["uc"], uc) and np.array_equal(d["om2"], om2) and np.array_equal(d["fnm1"], fnm1)
    assert d["om2"].dtype == np.complex64


def test_missing_file_and_wrong_container(tmp_path):
    with pytest.raises(FileNotFoundError):
        rs.read_restart_netcdf(str(tmp_path))
    with open(tmp_path / rs.RESTART_FILE, "wb") as f:
        f.write(b"\x89HDF\r\n\x1a\n" + b"\0" * 64)
    try:
        import netCDF4  # noqa: F401
        pytest.skip("netCDF4 is installed; the HDF5 path is the reference's own reader")
    except ImportError:
        pass
    with pytest.raises(RuntimeError, match="netCDF4"):
        rs.read_restart_netcdf(str(tmp_path))
    with open(tmp_path / rs.RESTART_FILE, "wb") as f:
        f.write(b"garbage!")
    with pytest.raises(RuntimeError, match="not a netCDF"):
        rs.read_restart_netcdf(str(tmp_path))


def test_wrong_field_shape_is_rejected(tmp_path):
    N = 16
    uc, om2, fnm1 = _fields(N)
    rs.write_restart_file(str(tmp_path / rs.RESTART_FILE), _attrs(N), uc, om2[:, :4], fnm1)
    with pytest.raises(ValueError, match="om2"):
        rs.read_restart_netcdf(str(tmp_path))


def test_compact_uc_layout():
    N = 16
    rng = np.random.default_rng(3)
    low = (rng.standard_normal((2, N, N // 2)) + 1j * rng.standard_normal((2, N, N // 2))).astype(np.complex64)
    uc = rs.uc_from_low_band(low, N)
    assert uc.shape == (N, 3 * N // 4 + 1, 3)
    assert np.array_equal(uc[:, : N // 2, 0], low[0]) and np.array_equal(uc[:, : N // 2, 1], low[1])
    assert not uc[:, N // 2:, :].any() and not uc[:, :, 2].any()
    assert np.array_equal(rs.low_band_from_uc(uc, N), low)
    with pytest.raises(ValueError):
        rs.low_band_from_uc(uc[:, :-1], N)


@pytest.mark.parametrize("N", [16, 64])
def test_velocity_from_om2_matches_oracle(N):
    """The save-side inversion agrees with the oracle's restatement of
    turbo_simulator.py:1555-1585 (FP32 arithmetic in both)."""
    rng = np.random.default_rng(N)
    om2 = (rng.standard_normal((N, N // 2)) + 1j * rng.standard_normal((N, N // 2))).astype(np.complex64)
    S = do.OracleState(N, om2, np.zeros((2, N, N // 2), np.complex64), 1e-4, 0.5, dtype=np.float32)
    do.reconstruct_velocity(S)
    got = rs.velocity_from_om2(om2)
    assert np.array_equal(got[0], S.uc_full[0, :N, : N // 2])
    assert np.array_equal(got[1], S.uc_full[1, :N, : N // 2])
