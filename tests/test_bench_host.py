"""bench.py's host-side helpers (no GPU): the roofline fields it reads from the
committed ncu summaries, and the reference arm's JSON line shape."""
import importlib.util
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_and_limiter_come_from_the_profiles(bench):
    t_row = bench._traffic("k_row", "fp32")
    t_col = bench._traffic("k_col", "fp32")
    assert t_row is not None and 3.0e8 < t_row < 5.0e8  # ~0.35 GB per N=4096 launch
    assert t_col is not None and 4.0e8 < t_col < 8.0e8  # 0.47-0.61 GB by RK3 stage
    lim = bench._limiter("k_row", "fp32")
    assert lim and "issue" in lim and "profiles/k_row_fp32_N4096.md" in lim
    assert bench._traffic("k_nonexistent", "fp32") is None


def test_rel_l2(bench):
    import numpy as np
    a = np.ones(4, np.complex64)
    assert bench._rel_l2(a, a) == 0.0
    assert abs(bench._rel_l2(2 * a, a) - 1.0) < 1e-12


def test_reference_arm_rank_nonzero_prints_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1"],
                         env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0
    assert out.stdout.strip() == ""


def test_warmup_is_raised_to_three(bench, monkeypatch, capsys):
    """The timing contract needs at least 3 warm-up steps; smaller values are raised."""
    seen = {}
    monkeypatch.setattr(bench, "run_reference", lambda args: seen.setdefault("warmup", args.warmup))
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--warmup", "1"])
    bench.main()
    assert seen["warmup"] == 3


def test_reference_arm_loads_nothing_from_the_product():
    """The reference arm builds its start with the oracle's restatement of the
    reference generator and times the oracle's FP32 port: palinstrophy_gb300
    (and its libpalgpu.so) is never imported."""
    code = (
        "import sys, types; sys.argv=['bench.py']; import bench; bench.N_GRID = 64; "
        "bench.run_reference(types.SimpleNamespace(steps=2, warmup=3, gpus=1)); "
        "bad = [m for m in sys.modules if m.startswith('palinstrophy_gb300')]; "
        "assert not bad, bad; print('CLEAN')")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[0])
    assert line["impl"] == "reference" and line["cpu_baseline"]["kind"] == "port"
    assert line["cpu_baseline"]["cores"] == min(8, os.cpu_count() or 1)
    assert line["warmup"] >= 3 and "3 warm-up steps" in line["cpu_baseline"]["sample"]
    assert out.stdout.strip().endswith("CLEAN")


def test_oracle_process_round_trip():
    """The spawned FP64 oracle leg returns the final field and the NEXTDT log
    (first row: the initial dt) of the same run done in-process."""
    import numpy as np
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench  # importable by name, as the spawned child needs
    from oracle import dns_oracle as do
    from oracle import pao_generator as pg
    g = pg.generate_fast(64, 10.0, 1e4, 4895, "KM3")
    run = bench._OracleRun(g["om2"], g["uc_low"], float(g["visc"]), 5)
    om2, log, secs, threads = run.result(timeout=300)
    S = do.OracleState(64, g["om2"], g["uc_low"], float(g["visc"]), bench.CFL)
    do.init_dt(S)
    dt0 = S.dt
    ref_log = []
    do.run(S, 5, bench.METHOD, bench.UPDATE, log=ref_log)
    assert np.array_equal(om2, S.om2)
    assert log[0, 0] == dt0 and len(log) == 1 + len(ref_log)
    assert [int(r[0]) for r in log[1:]] == [1, 5]
    assert secs > 0 and threads >= 1


def test_spectral_embedding_keeps_the_field():
    """The N=8192 comparison run starts from the N=4096 field embedded in the
    larger spectral grid: sampled on the coarse grid it is the same field."""
    import numpy as np
    import bench
    rng = np.random.default_rng(3)
    n, N = 32, 64
    om2 = (rng.standard_normal((n, n // 2)) + 1j * rng.standard_normal((n, n // 2))).astype(np.complex128)
    om2[n // 2, :] = 0.0                         # the kz = -n/2 row the n-grid step keeps at zero
    om2[0, 0] = om2[0, 0].real                   # Hermitian on the kx = 0 column
    om2[n - np.arange(1, n // 2), 0] = np.conj(om2[np.arange(1, n // 2), 0])
    big = bench._embed_spectrum(om2, N)
    assert big.shape == (N, N // 2)

    def field(c, m):
        full = np.zeros((m, m // 2 + 1), dtype=np.complex128)
        full[:, : c.shape[1]] = c
        return np.fft.irfft2(full, s=(m, m), norm="forward")

    small, large = field(om2, n), field(big, N)
    assert np.allclose(large[::2, ::2], small, atol=1e-12)
