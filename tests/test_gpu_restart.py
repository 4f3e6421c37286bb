"""Restart on the GPU state: save after some steps, load into a fresh handle,
continue.  With stale_uc=False the continued run equals the uninterrupted one
bit for bit (om2, fnm1, t, dt, cn, cnm1, it); with the reference's stale-uc
behaviour (default) the loaded physical velocity is the one of the saved
initial spectrum (turbo_main.py:1443-1445), while om2 / fnm1 are current."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ts(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from palinstrophy_gb300 import turbo_simulator
    return turbo_simulator


def _start(ts, N, method, precision="fp32"):
    S = ts.create_dns_state(N, 1e4, 10.0, 0.5, seed=4895, start_spectrum="KM3", precision=precision)
    ts._init_dt(S)
    S.field.set_scalar("it", 0)
    S.field.set_scalar("t", 0.0)
    return S


@pytest.mark.parametrize("method", ["CNAB2", "LS_IMEX_RK3"])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_restart_continues_exactly(ts, tmp_path, method, precision):
    from palinstrophy_gb300 import restart as rs
    N = 64
    S = _start(ts, N, method, precision)
    S.field.step(method, 12, update=5)
    if precision == "fp64":
        # the file stores float32 fields, as the reference does: round the state first
        S.set_spectral_state(S.om2.astype(np.complex64), S.fnm1.astype(np.complex64), None)
        ts.dns_step2a(S)
    rs.dump_restart_netcdf(S, str(tmp_path), stale_uc=False)
    S.field.step(method, 7, update=5)
    want = (S.om2, S.fnm1, S.field.scalars())

    L = rs.load_restart_netcdf(str(tmp_path), precision=precision, stale_uc=False)
    assert L.Nbase == N and L.seed_init == 4895 and L.start_spectrum == "KM3"
    L.field.step(method, 7, update=5)
    got = (L.om2, L.fnm1, L.field.scalars())
    assert np.array_equal(got[0], want[0])
    assert np.array_equal(got[1], want[1])
    for k in ("t", "dt", "cn", "cnm1", "visc", "cflnum", "it"):
        assert got[2][k] == want[2][k], k
    S.field.close()
    L.field.close()


def test_restart_stale_uc_mirrors_reference(ts, tmp_path):
    from palinstrophy_gb300 import restart as rs
    N = 64
    S = _start(ts, N, "CNAB2")
    u_init = S.field.ur(0).copy()
    S.field.step("CNAB2", 10, update=5)
    om_saved = S.om2
    rs.dump_restart_netcdf(S, str(tmp_path))  # stale: the generator's uc
    d = rs.read_restart_netcdf(str(tmp_path))
    assert np.array_equal(d["uc"], S.uc)
    assert d["it"] == 10

    L = rs.load_restart_netcdf(str(tmp_path))
    assert np.array_equal(L.om2, om_saved)
    # step2a ran on the stale spectrum: the physical velocity is the initial one
    assert np.array_equal(L.field.ur(0), u_init)
    # and saving the loaded state writes the same stale uc again
    rs.dump_restart_netcdf(L, str(tmp_path / "again"))
    assert np.array_equal(rs.read_restart_netcdf(str(tmp_path / "again"))["uc"], d["uc"])
    S.field.close()
    L.field.close()
