"""GPU parity: the sm_103a kernels against the CPU oracle, through the C ABI.

Tolerances (rel-L2 on the spectral vorticity om2 unless stated):
  FP64 path vs FP64 oracle : 1e-12 after 100 steps (1e-13 after one step)
  FP32 form vs FP64 oracle : 1e-4 after 100 steps
Both paths start from the identical initial arrays (the reference generator's
output, committed as fixtures) and compute their own CFL-adaptive dt; the dt
sequences are compared as well.
"""
import math

import numpy as np
import pytest

from conftest import golden
from oracle import dns_oracle as do
from oracle import pao_generator as pg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ts(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from palinstrophy_gb300 import turbo_simulator
    return turbo_simulator


def _init(name):
    d = golden(name)
    return d["om2"], d["uc_low"], float(d["visc"])


def _pair(ts, N, prec, om2, uc, visc, cfl):
    F = ts.Field(N, prec, 1e4, cfl)
    F.set_state(om2, None, uc)
    F.set_scalar("visc", visc)
    F.set_scalar("cflnum", cfl)
    S = do.OracleState(N, om2, uc, visc, cfl, dtype=np.float64)
    return F, S


def _gpu_init_dt(F):
    F.step2a()
    c = F.compute_cflm()
    dt = F.scalars()["cflnum"] / (c * math.pi)
    F.set_scalar("dt", dt)
    F.set_scalar("cn", 1.0)
    F.set_scalar("cnm1", 0.0)
    F.set_scalar("t", 0.0)
    F.set_scalar("it", 0)
    return c


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp32", 2e-6)])
@pytest.mark.parametrize("N,init", [(64, "init_KM3_N64_s4895_k10.npz"), (256, "init_KM3_N256_s4895_k10.npz")])
def test_initial_physical_field(ts, prec, tol, N, init):
    om2, uc, visc = _init(init)
    F, S = _pair(ts, N, prec, om2, uc, visc, 0.75)
    F.step2a()
    do.step2a(S)
    for c in (0, 1):
        ref = S.ur_full[c]
        got = F.ur(c).astype(np.float64)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < tol
    c_gpu, c_ref = F.compute_cflm(), do.compute_cflm(S)
    assert abs(c_gpu - c_ref) <= tol * c_ref
    F.close()


def _run_pair(ts, N, prec, init, cfl, method, steps, update):
    om2, uc, visc = _init(init)
    F, S = _pair(ts, N, prec, om2, uc, visc, cfl)
    c0g = _gpu_init_dt(F)
    c0 = do.init_dt(S)
    log = []
    do.run(S, steps, method, update, log=log)
    F.step(method, steps, update=update, final_update=True)
    return F, S, c0g, c0, log


@pytest.mark.parametrize("method,N,init,cfl,update", [
    ("CNAB2", 256, "init_KM3_N256_s4895_k10.npz", 0.75, 10),
    ("LS_IMEX_RK3", 128, "init_PAO_N128_s4895_k15.npz", 0.1, 25),
    ("CNAB2", 64, "init_KM3_N64_s4895_k10.npz", 0.75, 7),
])
def test_fp64_parity_100_steps(ts, method, N, init, cfl, update):
    F, S, c0g, c0, log = _run_pair(ts, N, "fp64", init, cfl, method, 100, update)
    assert abs(c0g - c0) <= 1e-14 * c0
    err_om = do.rel_l2(S.om2, F.om2())
    err_fn = do.rel_l2(S.fnm1, F.fnm1())
    sc = F.scalars()
    assert err_om <= 1e-12, err_om
    assert err_fn <= 1e-10, err_fn
    assert abs(sc["dt"] - S.dt) <= 1e-13 * S.dt
    assert abs(sc["cn"] - S.cn) <= 1e-13
    assert abs(sc["t"] - S.t) <= 1e-13 * S.t
    assert sc["it"] == 100
    F.close()


@pytest.mark.parametrize("method,N,init,cfl,update", [
    ("CNAB2", 256, "init_KM3_N256_s4895_k10.npz", 0.75, 10),
    ("LS_IMEX_RK3", 128, "init_PAO_N128_s4895_k15.npz", 0.1, 25),
])
def test_fp32_form_within_1e4(ts, method, N, init, cfl, update):
    F, S, _, _, _ = _run_pair(ts, N, "fp32", init, cfl, method, 100, update)
    err = do.rel_l2(S.om2, F.om2())
    assert err <= 1e-4, err
    assert abs(F.scalars()["dt"] - S.dt) <= 1e-5 * S.dt
    F.close()


def test_fp32_against_reference_fixture(ts):
    """FP32 form against the reference's own FP32 CPU run (fixture)."""
    d = golden("run_CNAB2_N256_s4895.npz")
    F = ts.Field(256, "fp32", 1e4, 0.75)
    F.set_state(d["om2_0"], None, d["uc_low_0"])
    F.set_scalar("visc", float(d["visc"]))
    _gpu_init_dt(F)
    F.step("CNAB2", 100, update=100, final_update=True)
    assert do.rel_l2(d["om2_100"], F.om2()) <= 1e-4
    F.close()


def test_diagnostics_match_oracle(ts):
    om2, uc, visc = _init("init_KM3_N256_s4895_k10.npz")
    F, S = _pair(ts, 256, "fp64", om2, uc, visc, 0.75)
    _gpu_init_dt(F)
    do.init_dt(S)
    F.step("CNAB2", 5, update=0)
    for _ in range(5):
        do.cnab2(S)
    d = F.diagnostics()
    U, Lh, tau = do.flow_eddy_metrics(S)
    sp = do.spectral_sums(S)
    assert abs(d["U"] - U) <= 1e-12 * U
    assert abs(d["L"] - Lh) <= 1e-12 * Lh
    assert abs(d["tau_l"] - tau) <= 1e-12 * tau
    for k in ("E", "Z", "P", "kmax2", "pal_over_ens_kmax2"):
        assert abs(d[k] - sp[k]) <= 1e-12 * abs(sp[k]), k
    assert abs(d["energy_joules"] - do.energy_joules(S)) <= 1e-12 * do.energy_joules(S)
    assert d["nonfinite"] == 0
    F.close()


@pytest.mark.parametrize("method", ["CNAB2", "LS_IMEX_RK3"])
def test_split_api_equals_fused_loop(ts, method):
    """dns_step2b/dns_step3/dns_step2a + next_dt == the fused pal_step loop, bit for bit."""
    om2, uc, visc = _init("init_KM3_N64_s4895_k10.npz")
    A = ts.Field(64, "fp64", 1e4, 0.5)
    B = ts.Field(64, "fp64", 1e4, 0.5)
    for F in (A, B):
        F.set_state(om2, None, uc)
        F.set_scalar("visc", visc)
        _gpu_init_dt(F)
    A.step(method, 20, update=5, final_update=True)
    for it in range(1, 21):
        if method == "CNAB2":
            B.step2b()
            B.step3()
            B.step2a()
        else:
            B.step_rk3()
        if it % 5 == 0 or it == 1:
            B.next_dt(sync_host=False)
    assert np.array_equal(A.om2(), B.om2())
    assert np.array_equal(A.fnm1(), B.fnm1())
    sa, sb = A.scalars(), B.scalars()
    assert sa["dt"] == sb["dt"] and sa["cn"] == sb["cn"]
    A.close()
    B.close()


SMALL = [32, 64, 128, 256, 384, 512, 768, 1024]


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp32", 5e-6)])
@pytest.mark.parametrize("N", SMALL)
def test_every_small_size_against_oracle(ts, prec, tol, N):
    """Every radix plan up to N=1024: 3 RK3 steps against the oracle."""
    g = pg.generate(N, 8.0, 1e4, 11, "KM3") if N <= 256 else None
    if g is None:
        from palinstrophy_gb300 import _lib as L
        om2, uc, st = L.pao_generate(N, 8.0, 1e4, 11, "KM3")
        visc = st["visc"]
    else:
        om2, uc, visc = g["om2"], g["uc_low"], float(g["visc"])
    F, S = _pair(ts, N, prec, om2, uc, visc, 0.3)
    _gpu_init_dt(F)
    do.init_dt(S)
    F.step("LS_IMEX_RK3", 3, update=1, final_update=True)
    do.run(S, 3, "LS_IMEX_RK3", update=1)
    assert do.rel_l2(S.om2, F.om2()) <= tol
    F.close()


@pytest.mark.parametrize("N", [2048, 3072, 4096])
def test_large_sizes_fp32_vs_fp64(ts, N):
    """Above the oracle's comfortable range: the FP32 and FP64 plans (different
    radix orders) must agree to FP32 accuracy, and the step must conserve the
    Parseval identity between physical and spectral energy."""
    from palinstrophy_gb300 import _lib as L
    om2, uc, st = L.pao_generate(N, 15.0, 1e5, 4895, "KM3")
    out = {}
    for prec in ("fp64", "fp32"):
        F = ts.Field(N, prec, 1e5, 0.1)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        _gpu_init_dt(F)
        F.step("LS_IMEX_RK3", 2, update=1, final_update=True)
        out[prec] = (F.om2().astype(np.complex128), F.diagnostics())
        F.close()
    assert do.rel_l2(out["fp64"][0], out["fp32"][0]) <= 2e-5
    d = out["fp64"][1]
    om = out["fp64"][0]
    nh = N // 2
    kx = np.arange(nh)[None, :]
    kz = np.fft.fftfreq(N, 1.0 / N)[:, None]
    k2 = kx * kx + kz * kz
    w = np.where(kx == 0, 1.0, 2.0)
    spec = float((w * np.abs(om) ** 2 / np.where(k2 > 0, k2, 1.0) * (k2 > 0)).sum())
    assert abs(d["U"] ** 2 - spec) <= 1e-6 * spec


def test_fp32_largest_grid_runs(ts):
    from palinstrophy_gb300 import _lib as L
    N = 8192
    om2, uc, st = L.pao_generate(N, 15.0, 1e5, 4895, "KM3")
    F = ts.Field(N, "fp32", 1e5, 0.1)
    F.set_state(om2, None, uc)
    F.set_scalar("visc", st["visc"])
    _gpu_init_dt(F)
    e0 = F.diagnostics()
    F.step("LS_IMEX_RK3", 2, update=1, final_update=True)
    e1 = F.diagnostics()
    assert e1["nonfinite"] == 0
    assert 0.9 * e0["U"] < e1["U"] <= 1.0001 * e0["U"]
    F.close()


def test_call_order_is_enforced(ts):
    from palinstrophy_gb300 import _lib as L
    om2, uc, visc = _init("init_KM3_N64_s4895_k10.npz")
    F = ts.Field(64, "fp32", 1e4, 0.5)
    with pytest.raises(L.PalError):
        F.step2b()  # no state yet
    F.set_state(om2, None, uc)
    with pytest.raises(L.PalError):
        F.step3()  # needs step2b first
    F.step2b()
    with pytest.raises(L.PalError):
        F.step2a()  # between step2b and step3
    F.step3()
    F.close()


def test_nonfinite_input_is_flagged(ts):
    om2, uc, visc = _init("init_KM3_N64_s4895_k10.npz")
    bad = om2.copy()
    bad[3, 4] = np.nan
    F = ts.Field(64, "fp64", 1e4, 0.5)
    F.set_state(bad, None, None)
    d = F.diagnostics()
    assert d["nonfinite"] == 1
    F.close()


def test_velocity_rebuilt_from_om2(ts):
    """Without uc_low the first step2a inverts om2 (restart path); it must match the
    generator's velocity to rounding, since both describe the same field."""
    om2, uc, visc = _init("init_KM3_N64_s4895_k10.npz")
    A = ts.Field(64, "fp64", 1e4, 0.5)
    A.set_state(om2, None, uc)
    B = ts.Field(64, "fp64", 1e4, 0.5)
    B.set_state(om2, None, None)
    A.step2a()
    B.step2a()
    ua, ub = A.ur(0), B.ur(0)
    assert np.linalg.norm(ua - ub) / np.linalg.norm(ua) < 1e-6
    A.close()
    B.close()


def test_dropin_run_dns(ts, capsys):
    S = ts.run_dns(N=64, Re=1e4, K0=10.0, STEPS=21, CFL=0.75, start_spectrum="KM3", UPDATE=10,
                   method="CNAB2", precision="fp64")
    out = capsys.readouterr().out
    assert "ITERATION     21" in out and "FPS" in out
    assert S.it == 21
    U, Lh, tau = S.flow_eddy_metrics()
    assert U > 0 and Lh > 0 and tau > 0


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp32", 2e-6)])
@pytest.mark.parametrize("N", [256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096, 8192])
def test_every_kernel_candidate_agrees(ts, prec, tol, N):
    """Each compiled row/column candidate (radix order, tile height, threads)
    gives the same field, so the autotuner's choice never changes results
    beyond rounding; at N <= 1024 the default candidates also match the oracle."""
    from palinstrophy_gb300 import _lib as L
    if not L.supported(N, prec):
        pytest.skip(f"{prec} is not compiled for N={N}")
    om2, uc, st = L.pao_generate(N, 12.0, 1e4, 7, "KM3")
    F = ts.Field(N, prec, 1e4, 0.3)
    v = F.variant()
    assert v["desc"].startswith("row[")
    F.set_state(om2, None, uc)
    F.step2a()
    dt = 0.3 / (F.compute_cflm() * math.pi)  # a stable step (CFL 0.3) at every N
    results = {}
    for r, c in [(r, 0) for r in range(v["n_rows"])] + [(0, c) for c in range(1, v["n_cols"])]:
        F.set_variant(r, c)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        F.set_scalar("dt", dt)
        F.set_scalar("cnm1", 0.0)
        F.step("LS_IMEX_RK3", 2, update=0)
        results[(r, c)] = F.om2().astype(np.complex128)
    ref = results[(0, 0)]
    for key, om in results.items():
        assert do.rel_l2(ref, om) <= tol, key
    if N <= 1024:
        S = do.OracleState(N, om2, uc, st["visc"], 0.3)
        do.step2a(S)
        S.dt = dt
        for _ in range(2):
            do.rk3(S)
        assert do.rel_l2(S.om2, ref) <= tol
    F.close()


@pytest.mark.parametrize("N,prec,tol", [(64, "fp64", 1e-12), (256, "fp64", 1e-12), (256, "fp32", 1e-6)])
def test_energy_spectrum_matches_oracle(ts, N, prec, tol):
    """Shell bins of |om|^2/K2 (GPU, deterministic) against the oracle's bincount."""
    from palinstrophy_gb300 import spectrum as sp
    g = pg.generate(N, 10.0, 1e4, 4895, "KM3") if N <= 64 else None
    if g is None:
        d = golden("init_KM3_N256_s4895_k10.npz")
        om2, uc, visc = d["om2"], d["uc_low"], float(d["visc"])
    else:
        om2, uc, visc = g["om2"], g["uc_low"], float(g["visc"])
    F, S = _pair(ts, N, prec, om2, uc, visc, 0.5)
    _gpu_init_dt(F)
    do.init_dt(S)
    F.step("CNAB2", 3, update=0)
    for _ in range(3):
        do.cnab2(S)
    s1 = sp.compute_energy_spectrum_uv_bins(F)
    s2 = sp.compute_energy_spectrum_uv_bins(F)
    assert np.array_equal(s1.energy, s2.energy)  # deterministic
    e_ref, c_ref = do.omega_spectrum_bins(S)
    assert np.array_equal(s1.count, c_ref)
    m = e_ref > 0
    if prec == "fp64":  # every bin to double rounding
        assert np.max(np.abs(s1.energy[m] - e_ref[m]) / e_ref[m]) <= tol
    else:  # FP32 field: the spectrum as a whole
        assert np.abs(s1.energy - e_ref).sum() / e_ref.sum() <= tol
    assert s1.nbins == max(32, 2 * N)
    F.close()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-6)])
def test_display_fields_match_oracle(ts, prec, tol):
    """u, v, |u|, omega, streamfunction on the 3/2 grid and their 8-bit frames;
    the display passes must leave the simulation state untouched."""
    om2, uc, visc = _init("init_KM3_N64_s4895_k10.npz")
    F, S = _pair(ts, 64, prec, om2, uc, visc, 0.5)
    _gpu_init_dt(F)
    do.init_dt(S)
    F.step("CNAB2", 4, update=0)
    for _ in range(4):
        do.cnab2(S)
    before = F.om2()
    refs = {0: S.ur_full[0], 1: S.ur_full[1], 2: do.kinetic(S), 3: do.om2_phys(S), 4: do.stream_func(S)}
    for var, ref in refs.items():
        f, pix = F.vis(var, field=True, pixels=True)
        err = np.linalg.norm(f.astype(np.float64) - ref) / np.linalg.norm(ref)
        assert err <= tol, (var, err)
        rp = do.to_pixels(ref)
        assert np.mean(np.abs(pix.astype(int) - rp.astype(int)) <= 1) > 0.999, var
    assert np.array_equal(before, F.om2())
    d = F.diagnostics()
    U, _, _ = do.flow_eddy_metrics(S)
    assert abs(d["U"] - U) <= 1e-5 * U
    F.close()


def test_k4_start_runs(ts):
    from palinstrophy_gb300.initial import k4_unit_energy
    om2, uc = k4_unit_energy(256, 15.0, 4895)
    F = ts.Field(256, "fp32", 1e4, 0.1)
    F.set_state(om2, None, uc)
    F.set_scalar("visc", 1e-4)
    _gpu_init_dt(F)
    d0 = F.diagnostics()
    # Parseval: mean(u^2 + v^2) on the 3/2 grid equals the unit energy measure
    assert abs(d0["U"] ** 2 - 1.0) < 1e-5
    F.step("LS_IMEX_RK3", 5, update=1, final_update=True)
    assert F.diagnostics()["nonfinite"] == 0
    F.close()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_device_views_match_host_copies(ts, prec):
    """__cuda_array_interface__ views of om2 / fnm1 (strided: the device keeps them
    [kx][z]) and of the physical u, v planes read the same values as the copies."""
    import torch
    from palinstrophy_gb300 import _lib as L
    om2, uc, st = L.pao_generate(64, 10.0, 1e4, 4895, "KM3")
    F = ts.Field(64, prec, 1e4, 0.5)
    F.set_state(om2, None, uc)
    F.set_scalar("visc", st["visc"])
    F.step2a()
    F.set_scalar("dt", 1e-3)
    F.step("CNAB2", 3, update=0)
    F.synchronize()
    for name, host in (("om2", F.om2()), ("fnm1", F.fnm1())):
        t = torch.as_tensor(F.device_array(name), device="cuda")
        assert t.shape == host.shape
        assert np.array_equal(t.cpu().numpy(), host)
    u = torch.as_tensor(F.device_array("u"), device="cuda")
    F.synchronize()
    assert np.array_equal(u.cpu().numpy(), F.ur(0))
    F.close()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-4)])
def test_precision_form_config_n1024(ts, prec, tol):
    """The precision-form configuration at its own size: N=1024 from the labelled
    k^4 unit-energy start (K0=15, seed 4895), Re=1e4, LS-IMEX-RK3 at CFL 0.1,
    NEXTDT every 10 steps; 20 steps against the FP64 oracle."""
    from palinstrophy_gb300.initial import k4_unit_energy
    N, cfl, steps, update = 1024, 0.1, 20, 10
    om2, uc = k4_unit_energy(N, 15.0, 4895)
    visc = float(np.float32(1.0 / np.float32(1e4)))
    F, S = _pair(ts, N, prec, om2, uc, visc, cfl)
    _gpu_init_dt(F)
    do.init_dt(S)
    do.run(S, steps, "LS_IMEX_RK3", update)
    F.step("LS_IMEX_RK3", steps, update=update, final_update=True)
    err = do.rel_l2(S.om2, F.om2())
    assert err <= tol, err
    assert abs(F.scalars()["dt"] - S.dt) <= (1e-13 if prec == "fp64" else 1e-5) * S.dt
    F.close()


def test_reference_plain_config_blows_up_like_the_reference(ts):
    """The plain CPU configuration (N=256 KM3 K0=10 seed 4895, Re=1e4, CNAB2,
    CFL 0.75, NEXTDT every 100 steps) is unstable: the reference's own run_dns
    turns non-finite between steps 200 and 300 (ITERATION 300 prints DT=nan).
    The FP64 path follows the oracle up to step 200 and then turns non-finite
    with it, and the diagnostics flag it."""
    om2, uc, visc = _init("init_KM3_N256_s4895_k10.npz")
    for steps, finite in ((200, True), (300, False)):
        F, S, _, _, _ = _run_pair(ts, 256, "fp64", "init_KM3_N256_s4895_k10.npz", 0.75, "CNAB2", steps, 100)
        if finite:
            assert np.isfinite(S.om2).all()
            assert do.rel_l2(S.om2, F.om2()) <= 1e-9
        else:
            assert not np.isfinite(S.om2).all()
            assert not np.isfinite(F.om2()).all()
            assert F.diagnostics()["nonfinite"] != 0
        F.close()


@pytest.mark.parametrize("method", ["CNAB2", "LS_IMEX_RK3"])
def test_step_graph_replay_equals_direct_launches(ts, method, monkeypatch):
    """Small grids replay pal_step sequences from CUDA graphs (one per NEXTDT
    pattern); the replayed steps equal directly launched ones bit for bit."""
    from palinstrophy_gb300 import _lib as L
    om2, uc, st = L.pao_generate(128, 12.0, 1e4, 4895, "KM3")
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("PAL_STEP_GRAPHS", mode)
        F = ts.Field(128, "fp32", 1e4, 0.5)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        _gpu_init_dt(F)
        for _ in range(3):  # the same pattern three times: captured once, replayed twice
            F.step(method, 10, update=5)
        out[mode] = (F.om2(), F.scalars())
        F.close()
    assert np.array_equal(out["1"][0], out["0"][0])
    for k in ("t", "dt", "cn", "cnm1", "it"):
        assert out["1"][1][k] == out["0"][1][k], k


def test_two_row_tiles_share_an_sm(ts):
    """The 2-row FP32 row tiles at N=4096 (102.4 KB of shared memory each) are
    built to run two per SM; the occupancy calculator must agree, so a register
    budget that grows past the cap shows up here and not only as a slower step."""
    from palinstrophy_gb300 import _lib as L
    if not L.supported(4096, "fp32"):
        pytest.skip("fp32 is not compiled for N=4096")
    F = ts.Field(4096, "fp32", 1e5, 0.1)
    v = F.variant()
    assert v["row_blocks_per_sm"] >= 1 and v["col_blocks_per_sm"] >= 1
    seen = 0
    for r in range(v["n_rows"]):
        F.set_variant(r, v["col"])
        w = F.variant()
        if "V2x384" in w["desc"]:
            seen += 1
            assert w["row_blocks_per_sm"] == 2, w["desc"]
    assert seen >= 2
    F.close()


def test_tma_column_pass_equals_per_lane_column_pass(ts):
    """The column pass that moves its planes by TMA into a planar padded tile
    (`... tma`) does the per-lane kernel's arithmetic in the same order, so on
    the same plan and block size the fields agree bit for bit."""
    from palinstrophy_gb300 import _lib as L
    N = 1024
    if not L.supported(N, "fp32"):
        pytest.skip("fp32 is not compiled for N=1024")
    om2, uc, st = L.pao_generate(N, 12.0, 1e4, 5, "KM3")
    F = ts.Field(N, "fp32", 1e4, 0.3)
    v = F.variant()
    cols = {}
    for c in range(v["n_cols"]):
        F.set_variant(v["row"], c)
        cols[F.variant()["desc"].split("col[")[1].rstrip("]")] = c
    assert "16.4.24r x128 tma" in cols and "16.4.24r x128 pref" in cols
    out = []
    for name in ("16.4.24r x128 pref", "16.4.24r x128 tma"):
        F.set_variant(v["row"], cols[name])
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        F.step2a()
        F.set_scalar("dt", 0.3 / (F.compute_cflm() * math.pi))
        F.set_scalar("cn", 1.0)
        F.set_scalar("cnm1", 0.0)
        for method in ("LS_IMEX_RK3", "CNAB2"):
            F.step(method, 3, update=0)
        out.append((F.om2(), F.fnm1()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    F.close()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_diagnostic_sums_are_compensated_fp64(ts, prec):
    """The diagnostic sums run in FP64 with compensated (TwoSum) accumulation in
    both precisions: on the FP32 form's own field (N=1024, 20 RK3 steps) the GPU's
    E, Z, P and mean(u^2 + v^2) equal the FP64 oracle's sums over the same values
    -- the downloaded om2 and physical planes, which the diagnostics kernels read
    -- to 1e-10 relative (turbo_simulator.py:764-810, turbo_main.py:2015-2073)."""
    from palinstrophy_gb300 import _lib as L
    N = 1024
    om2, uc, st = L.pao_generate(N, 15.0, 1e4, 4895, "KM3")
    F = ts.Field(N, prec, 1e4, 0.1)
    F.set_state(om2, None, uc)
    F.set_scalar("visc", st["visc"])
    _gpu_init_dt(F)
    F.step("LS_IMEX_RK3", 20, update=10, final_update=True)
    d = F.diagnostics()
    om, u, v = F.om2(), F.ur(0), F.ur(1)
    S = do.OracleState(N, om.astype(np.complex128), np.zeros((2, N, N // 2), np.complex128), st["visc"], 0.1)
    S.ur_full[0] = u.astype(np.float64)
    S.ur_full[1] = v.astype(np.float64)
    U, _, _ = do.flow_eddy_metrics(S)
    sp = do.spectral_sums(S)
    assert abs(d["U"] ** 2 / U ** 2 - 1.0) <= 1e-10
    for k in ("E", "Z", "P"):
        assert abs(d[k] / sp[k] - 1.0) <= 1e-10, (k, d[k], sp[k])
    F.close()


def test_multicast_candidates_can_be_left_out(ts):
    """PAL_TMA_MULTICAST=0 keeps the autotuner off the row candidates that load
    by TMA cluster multicast (read when a size is first tuned in a process,
    hence a fresh interpreter)."""
    import os
    import subprocess
    import sys
    from palinstrophy_gb300 import _lib as L
    if not L.supported(8192, "fp32"):
        pytest.skip("fp32 is not compiled for N=8192")
    code = ("from palinstrophy_gb300.turbo_simulator import Field\n"
            "F = Field(8192, 'fp32', 1e5, 0.1)\n"
            "print(F.variant()['desc'])\n"
            "F.close()\n")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, check=True,
                         env={**os.environ, "PAL_TMA_MULTICAST": "0"}, timeout=600)
    desc = out.stdout.strip().splitlines()[-1]
    assert desc.startswith("row[") and " mc " not in desc, desc


def test_tuning_file_pins_the_candidates(ts, tmp_path):
    """PAL_TUNE_FILE: a size listed there takes the named candidates without
    timing, a size that is timed is appended, and a later process reading the
    file runs the same kernels."""
    import os
    import subprocess
    import sys
    F = ts.Field(128, "fp32", 1e4, 0.5)
    F.set_variant(1, 1)
    want = F.variant()["desc"]
    F.close()
    rname = want.split("row[")[1].split("]")[0]
    cname = want.split("col[")[1].split("]")[0]
    tf = tmp_path / "tune.txt"
    tf.write_text(f"# comment lines and other sizes are skipped\nfp64 128 {rname}|{cname}\nfp32 128 {rname}|{cname}\n")
    code = ("from palinstrophy_gb300.turbo_simulator import Field\n"
            "for n in (128, 64):\n"
            "    F = Field(n, 'fp32', 1e4, 0.5)\n"
            "    print(F.variant()['desc'])\n"
            "    F.close()\n")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {**os.environ, "PAL_TUNE_FILE": str(tf)}
    env.pop("PAL_AUTOTUNE", None)

    def run():
        out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, check=True,
                             env=env, timeout=600)
        return out.stdout.strip().splitlines()[-2:]

    first = run()
    assert first[0] == want
    lines = tf.read_text().splitlines()
    assert len(lines) == 4 and lines[3].startswith("fp32 64 "), lines
    assert run() == first
    assert len(tf.read_text().splitlines()) == 4  # nothing timed the second time
