"""The device generator (pal_generate) against the reference's own initial
fields (committed fixtures) and against the host restatement.  Float32
exp/sin/cos (and double sin/cos) come from CUDA's library here, from NumPy in
the reference and libm in the host restatement, so values agree to a few ulp,
as the host restatement's do; seeds, shells and the mode set are exact."""
import platform

import numpy as np
import pytest

from conftest import golden
from oracle import pao_generator as pg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ts(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from palinstrophy_gb300 import turbo_simulator
    return turbo_simulator


def _gen(ts, N, K0, Re, seed, spec, prec="fp32"):
    F = ts.Field(N, prec, Re, 0.5)
    uc, st = F.generate(K0, Re, seed, spec)
    om2 = F.om2()
    F.close()
    return om2, uc, st


@pytest.mark.parametrize("name,N,K0,seed,spec", [
    ("init_KM3_N64_s4895_k10.npz", 64, 10.0, 4895, "KM3"),
    ("init_KM3_N128_s4895_k15.npz", 128, 15.0, 4895, "KM3"),
    ("init_KM3_N256_s4895_k10.npz", 256, 10.0, 4895, "KM3"),
    ("init_PAO_N128_s4895_k15.npz", 128, 15.0, 4895, "PAO"),
    ("init_PAO_N64_s7_k12.npz", 64, 12.0, 7, "PAO"),
])
def test_device_generator_matches_reference_fixture(ts, name, N, K0, seed, spec):
    d = golden(name)
    om2, uc, st = _gen(ts, N, K0, 1e4, seed, spec)
    assert st["seed_out"] == int(d["seed_out"])
    scale_u = np.abs(d["uc_low"]).max()
    assert np.abs(uc - d["uc_low"]).max() <= 4e-7 * scale_u
    assert np.abs(om2 - d["om2"]).max() <= 4e-7 * np.abs(d["om2"]).max()
    assert abs(st["Energy"] - float(d["Energy"])) <= 1e-6 * max(1.0, float(d["Energy"]))
    assert np.float32(st["visc"]) == np.float32(d["visc"])
    # the mode set is exact: zeros where the reference has zeros
    assert np.array_equal(uc == 0, d["uc_low"] == 0)


@pytest.mark.parametrize("spec", ["KM3", "PAO"])
def test_device_generator_matches_host_generator(ts, spec):
    from palinstrophy_gb300 import _lib as L
    N, K0, Re, seed = 1024, 15.0, 1e5, 4895
    om2, uc, st = _gen(ts, N, K0, Re, seed, spec)
    om2_h, uc_h, st_h = L.pao_generate(N, K0, Re, seed, spec)
    assert st["seed_out"] == st_h["seed_out"]
    assert np.abs(uc - uc_h).max() <= 4e-7 * np.abs(uc_h).max()
    assert np.abs(om2 - om2_h).max() <= 4e-7 * np.abs(om2_h).max()
    assert abs(st["Energy"] / st_h["Energy"] - 1.0) < 1e-6
    assert abs(st["WiWi"] / st_h["WiWi"] - 1.0) < 1e-6


def test_device_generator_oracle_restatement_small(ts):
    """Against the oracle's restatement of the generator at a size it runs in seconds."""
    g = pg.generate(32, 6.0, 1e4, 11, "KM3")
    om2, uc, st = _gen(ts, 32, 6.0, 1e4, 11, "KM3")
    assert st["seed_out"] == g["seed_out"]
    assert np.abs(uc - g["uc_low"]).max() <= 4e-7 * np.abs(g["uc_low"]).max()


def test_fp64_handle_gets_the_same_start(ts):
    om32, uc32, _ = _gen(ts, 128, 15.0, 1e4, 4895, "KM3", "fp32")
    om64, uc64, _ = _gen(ts, 128, 15.0, 1e4, 4895, "KM3", "fp64")
    assert np.array_equal(om64, om32.astype(np.complex128))
    assert np.array_equal(uc64, uc32.astype(np.complex128))


@pytest.mark.parametrize("name", ["init_KM3_N64_s4895_k10", "init_KM3_N128_s4895_k15", "init_KM3_N256_s4895_k10",
                                  "init_PAO_N128_s4895_k15", "init_PAO_N64_s7_k12"])
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_create_dns_state_starts_from_the_reference_field(ts, name, prec):
    """The default create_dns_state path holds the reference generator's arrays as
    the reference computes them on this machine: bit for bit equal to the oracle's
    scalar restatement of the generator (NumPy float32 scalars, as the reference)
    run here.  The fixtures were made by the reference on x86-64, and NumPy's
    float32 cos/sin/exp kernels differ between CPU architectures in the last bit,
    so against them the arrays are bit-exact on x86-64 (also checked without a GPU
    in tests/test_abi.py) and within a few ulp elsewhere."""
    d = golden(name + ".npz")
    N = int(d["N"])
    S = ts.create_dns_state(N, float(d["Re"]), float(d["K0"]), 0.5, seed=int(d["seed"]),
                            start_spectrum=str(d["spectrum"]), precision=prec)
    om2 = S.om2
    g = pg.generate(N, float(d["K0"]), float(d["Re"]), int(d["seed"]), str(d["spectrum"]))
    assert np.array_equal(om2, g["om2"].astype(om2.dtype))
    assert np.array_equal(S.uc_init.view(np.uint32), g["uc_low"].view(np.uint32))
    if platform.machine() in ("x86_64", "AMD64"):
        assert np.array_equal(S.uc_init.view(np.uint32), d["uc_low"].view(np.uint32))
    else:
        assert np.abs(S.uc_init - d["uc_low"]).max() <= 4e-7 * np.abs(d["uc_low"]).max()
        assert np.abs(om2 - d["om2"]).max() <= 4e-7 * np.abs(d["om2"]).max()
    assert S.visc == float(d["visc"])
    S.field.close()


def test_create_dns_state_device_generator_steps(ts):
    S = ts.create_dns_state(128, 1e4, 15.0, 0.5, seed=4895, start_spectrum="KM3", generator="device")
    ts._init_dt(S)
    S.field.step("LS_IMEX_RK3", 5, update=1)
    d = S.diagnostics()
    assert np.isfinite(d["E"]) and d["E"] > 0
    assert S.uc.shape == (128, 97, 3)
    S.field.close()


def test_generator_rejects_bad_arguments(ts):
    F = ts.Field(64, "fp32", 1e4, 0.5)
    with pytest.raises(KeyError):
        F.generate(10.0, 1e4, 1, "XYZ")
    with pytest.raises(ValueError):
        F.generate(-1.0, 1e4, 1, "KM3")
    F.close()


def test_reading_om2_keeps_a_pending_velocity_band(ts):
    """om2() between the velocity upload and STEP2A must not disturb the band
    (the getter's scratch buffer is where the band waits)."""
    from palinstrophy_gb300 import _lib as L
    om2, uc, st = L.pao_generate(64, 10.0, 1e4, 4895, "KM3")
    A = ts.Field(64, "fp32", 1e4, 0.5)
    A.set_state(om2, None, uc)
    A.step2a()
    ref = A.ur(0).copy()
    B = ts.Field(64, "fp32", 1e4, 0.5)
    B.set_state(om2, None, uc)
    _ = B.om2()
    B.step2a()
    assert np.array_equal(B.ur(0), ref)
    C = ts.Field(64, "fp32", 1e4, 0.5)
    C.generate(10.0, 1e4, 4895, "KM3")
    _ = C.om2()
    C.step2a()
    D = ts.Field(64, "fp32", 1e4, 0.5)
    D.generate(10.0, 1e4, 4895, "KM3")
    D.step2a()
    assert np.array_equal(C.ur(0), D.ur(0))
    for F in (A, B, C, D):
        F.close()
