"""The CPU oracle pinned against fixtures generated from the reference itself.

tests/golden/make_golden.py ran the reference's own generator and FP32 CPU
step functions; these tests check that the oracle restatement reproduces them
(bit for bit where the arithmetic allows) before the oracle is trusted as the
checker of the GPU path.
"""
import os

import numpy as np
import pytest

from conftest import golden
from oracle import dns_oracle as do
from oracle import pao_generator as pg

INITS = ["init_KM3_N64_s4895_k10", "init_KM3_N128_s4895_k15", "init_PAO_N64_s7_k12",
         "init_PAO_N128_s4895_k15"]


@pytest.mark.parametrize("name", INITS)
def test_generator_bit_exact(name):
    d = golden(name + ".npz")
    g = pg.generate(int(d["N"]), float(d["K0"]), float(d["Re"]), int(d["seed"]), str(d["spectrum"]))
    assert np.array_equal(g["om2"], d["om2"])
    assert np.array_equal(g["uc_low"], d["uc_low"])
    assert g["seed_out"] == int(d["seed_out"])
    assert abs(g["Q2"] - float(d["Energy"])) <= 1e-7 * abs(float(d["Energy"]))
    assert abs(g["W2"] - float(d["WiWi"])) <= 1e-6 * abs(float(d["WiWi"]))
    assert g["visc"] == d["visc"]


@pytest.mark.parametrize("name", INITS + ["init_KM3_N256_s4895_k10"])
def test_fast_generator_bit_exact(name):
    """The vectorised restatement gives the fixtures bit for bit (signs of zeros too)."""
    d = golden(name + ".npz")
    g = pg.generate_fast(int(d["N"]), float(d["K0"]), float(d["Re"]), int(d["seed"]), str(d["spectrum"]))
    assert np.array_equal(g["om2"].view(np.uint32), d["om2"].view(np.uint32))
    assert np.array_equal(g["uc_low"].view(np.uint32), d["uc_low"].view(np.uint32))
    assert g["seed_out"] == int(d["seed_out"])


@pytest.mark.parametrize("N,K0,seed,spec", [(96, 12.0, 7, "KM3"), (160, 6.0, 11, "PAO"), (200, 20.0, 5010, "KM3")])
def test_fast_generator_equals_scalar_restatement(N, K0, seed, spec):
    a = pg.generate(N, K0, 1e4, seed, spec)
    b = pg.generate_fast(N, K0, 1e4, seed, spec)
    for k in ("om2", "uc_low"):
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    assert a["seed_out"] == b["seed_out"] and a["Q2"] == b["Q2"] and a["W2"] == b["W2"]


def test_generator_known_answer_N256():
    """The printed init KAT: N=256 KM3 seed 4895 -> Energy 0.99681688, WiWi 384.68516, seed 4983."""
    d = golden("init_KM3_N256_s4895_k10.npz")
    assert abs(float(d["Energy"]) - 0.99681688) < 1e-8
    assert abs(float(d["WiWi"]) - 384.68516) < 1e-5
    assert int(d["seed_out"]) == 4983
    g = pg.generate(256, 10.0, 1e4, 4895, "KM3")
    assert np.array_equal(g["om2"], d["om2"])


def _run(d, dtype, replay):
    N = int(d["N"])
    S = do.OracleState(N, d["om2_0"], d["uc_low_0"], d["visc"], float(d["cfl"]), dtype=dtype)
    cflm0 = do.init_dt(S)
    step = do.rk3 if str(d["method"]) == "LS_IMEX_RK3" else do.cnab2
    log = d["log"]
    snaps, mylog, nd = {}, [], 0
    steps, upd = int(d["steps"]), int(d["update"])
    for it in range(1, steps + 1):
        dt_old = S.dt
        step(S)
        if it % upd == 0 or it == 1 or it == steps:
            c = do.next_dt(S)
            mylog.append((it, S.t, S.dt, S.cn, c))
            if replay:
                S.dt, S.cn = float(log[nd][2]), float(log[nd][3])
            nd += 1
        S.t += dt_old
        if it in (1, 10, steps):
            snaps[it] = (S.om2.copy(), S.fnm1.copy())
    return cflm0, np.array(mylog), snaps


RUNS = ["run_CNAB2_N64_s4895", "run_LS_IMEX_RK3_N64_s4895", "run_LS_IMEX_RK3_N128_s4895",
        "run_CNAB2_N256_s4895"]


@pytest.mark.parametrize("name", RUNS)
def test_fp32_port_matches_reference(name):
    """FP32 mode follows the reference CPU path operation for operation.

    pocketfft batches lines per worker count, so it is bit-exact at the
    reference's own worker count min(8, cpu_count) = 8 (the fixtures' host)."""
    d = golden(name + ".npz")
    cflm0, log, snaps = _run(d, np.float32, replay=False)
    assert cflm0 == float(d["cflm0"])
    exact = (os.cpu_count() or 1) >= 8
    for it, (o, f) in snaps.items():
        if exact:
            assert np.array_equal(o, d[f"om2_{it}"]), f"om2 differs at it={it}"
            assert np.array_equal(f, d[f"fnm1_{it}"])
        else:
            assert do.rel_l2(d[f"om2_{it}"], o) < 1e-5
    np.testing.assert_allclose(log[:, 2], d["log"][:, 2], rtol=0 if exact else 1e-6)


@pytest.mark.parametrize("name", RUNS)
def test_fp64_oracle_vs_reference_fp32(name):
    """FP64 oracle against the reference's FP32 path, dt sequence replayed: FP32 error level."""
    d = golden(name + ".npz")
    _, _, snaps = _run(d, np.float64, replay=True)
    for it, (o, f) in snaps.items():
        assert do.rel_l2(d[f"om2_{it}"], o) < 3e-5, it
        assert do.rel_l2(d[f"fnm1_{it}"], f) < 1e-4, it


def test_oracle_flow_metrics_match_reference_log():
    """U/L printed by the reference at each NEXTDT agree with the FP64 oracle's."""
    d = golden("run_CNAB2_N64_s4895.npz")
    N = 64
    S = do.OracleState(N, d["om2_0"], d["uc_low_0"], d["visc"], float(d["cfl"]))
    do.init_dt(S)
    do.cnab2(S)
    do.next_dt(S)
    U, Lh, tau = do.flow_eddy_metrics(S)
    row = d["log"][0]
    assert abs(U - row[5]) < 1e-5 * row[5]
    assert abs(Lh - row[6]) < 1e-5 * row[6]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_threaded_passes_equal_single_thread(dtype):
    """The elementwise passes split over host threads give the same bits as one thread."""
    N = 512
    d = golden("init_KM3_N256_s4895_k10.npz")
    rng = np.random.default_rng(3)
    om2 = np.zeros((N, N // 2), np.complex64)
    om2[:128, :128] = d["om2"][:128, :128]
    om2[-128:, :128] = d["om2"][-128:, :128]
    om2 += (1e-3 * (rng.standard_normal(om2.shape) + 1j * rng.standard_normal(om2.shape))).astype(np.complex64)
    om2[0, 0] = 0
    runs = []
    for threads in (1, 8):
        S = do.OracleState(N, om2, np.zeros((2, N, N // 2), np.complex64), d["visc"], 0.5, dtype=dtype,
                           threads=threads)
        do.reconstruct_velocity(S)
        do.init_dt(S)
        do.rk3(S)
        do.cnab2(S)
        runs.append((S.om2, S.fnm1, S.ur_full))
    for a, b in zip(*runs):
        assert np.array_equal(a, b)
