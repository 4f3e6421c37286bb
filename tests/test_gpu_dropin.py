"""The drop-in state through the reference GUI facade's call sequence.

DnsSimulator.make_pixels_component (turbo_wrapper.py:420-470) reads the
velocity planes straight from S.ur_full[0] / S.ur_full[1], and for the energy,
vorticity and streamfunction views calls dns_kinetic / dns_om2_phys /
dns_stream_func and then reads S.ur_full[2]; frames are 8-bit grey levels
1..255 (turbo_wrapper.py:317-351).  The sequence is replayed here on a
create_dns_state(backend="gb300") state and compared with the oracle's fields.
"""
import numpy as np
import pytest

from oracle import dns_oracle as do

pytestmark = pytest.mark.gpu

VAR_U, VAR_V, VAR_ENERGY, VAR_OMEGA, VAR_STREAM = 1, 2, 3, 4, 5   # the facade's selector values


@pytest.fixture(scope="module")
def ts(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from palinstrophy_gb300 import turbo_simulator
    return turbo_simulator


def _make_pixels_component(ts, S, var):
    """The CPU-side branch of turbo_wrapper.py:436-470 (backend != "gpu")."""
    if var == VAR_U:
        field = np.asarray(S.ur_full[0, :, :])
    elif var == VAR_V:
        field = np.asarray(S.ur_full[1, :, :])
    else:
        helper = {VAR_ENERGY: ts.dns_kinetic, VAR_OMEGA: ts.dns_om2_phys, VAR_STREAM: ts.dns_stream_func}[var]
        helper(S)
        field = np.asarray(S.ur_full[2, :, :])
    return field, do.to_pixels(field)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-6)])
def test_make_pixels_component_sequence(ts, prec, tol, capsys):
    N = 64
    S = ts.create_dns_state(N, 1e4, 10.0, 0.5, seed=4895, start_spectrum="KM3", precision=prec)
    O = do.OracleState(N, S.om2, S.uc_init, S.visc, 0.5)
    ts._init_dt(S)
    do.init_dt(O)
    for _ in range(3):
        ts.dns_step2b(S)
        ts.dns_step3(S)
        ts.dns_step2a(S)
        do.cnab2(O)
    refs = {VAR_U: O.ur_full[0], VAR_V: O.ur_full[1], VAR_ENERGY: do.kinetic(O), VAR_OMEGA: do.om2_phys(O),
            VAR_STREAM: do.stream_func(O)}
    for var in (VAR_U, VAR_ENERGY, VAR_V, VAR_OMEGA, VAR_STREAM, VAR_U):
        field, pix = _make_pixels_component(ts, S, var)
        ref = refs[var]
        assert do.rel_l2(ref, field) <= tol, var
        rp = do.to_pixels(ref)
        assert np.mean(np.abs(pix.astype(int) - rp.astype(int)) <= 1) > 0.999, var
        assert len(np.unique(pix)) > 50, var          # a real image, not a blank frame
    # the display plane is the last helper's output and stays until the next helper
    stream = np.array(S.ur_full[2])
    ts.dns_step2b(S)
    ts.dns_step3(S)
    ts.dns_step2a(S)
    assert np.array_equal(np.asarray(S.ur_full[2]), stream)
    do.cnab2(O)
    assert do.rel_l2(O.ur_full[0], np.asarray(S.ur_full[0])) <= tol   # velocity planes follow the step
    S.field.close()


def test_energy_joules_reads_planes_without_extra_copies(ts, monkeypatch):
    """energy_joules (turbo_main.py:1947-1959) reads ur_full[0] and ur_full[1]:
    one device copy per plane per state change, however often they are read."""
    S = ts.create_dns_state(64, 1e4, 10.0, 0.5, seed=4895, start_spectrum="KM3", precision="fp64")
    ts._init_dt(S)
    calls = []
    real = S.field.ur_into
    monkeypatch.setattr(S.field, "ur_into", lambda c, out: (calls.append(c), real(c, out))[1])
    for _ in range(3):
        u = S.ur_full[0]
        v = S.ur_full[1]
        e = 0.5 * (2 * np.pi) ** 2 * float((u.astype(np.float64) ** 2 + v.astype(np.float64) ** 2).mean())
    assert calls == [0, 1]
    d = S.diagnostics()
    assert abs(d["energy_joules"] - e) <= 1e-12 * e
    S.field.step("CNAB2", 1)
    _ = S.ur_full[0]
    assert calls == [0, 1, 0]
    S.field.close()
