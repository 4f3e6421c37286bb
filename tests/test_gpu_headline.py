"""The headline configuration against the FP64 oracle, at the sizes the bench runs.

N=4096 (3/2-padded 6144^2), KM3 K0=15 seed 4895, Re=1e5, LS-IMEX-RK3, CFL 0.1,
NEXTDT after step 1 and every 100 steps (turbo_simulator.py:1900-1943 stage,
2127-2167 NEXTDT, 2831-2848 cadence), 100 steps.  The oracle runs the FP64 CPU
restatement once; its dt / cn sequence is replayed into every GPU run, so the
comparison measures the step's arithmetic alone:

  FP64 GPU path vs FP64 oracle : rel-L2 <= 1e-12 on om2 after 100 steps
  FP32 form     vs FP64 oracle : rel-L2 <= 1e-4 after 100 steps, for every
                                 compiled row and column kernel candidate
  the GPU's own NEXTDT after step 1 (CFLM, dt, cn) vs the oracle's: 1e-12 FP64

N=2048 (the TMA column and row candidates at a second size), 10 steps, the
same checks.  N=8192 (padded 12288^2, FP32 only: the cluster-split row passes
and every other candidate), 3 steps against the FP64 oracle.  The oracle
costs a few seconds per step at N=4096 and N=8192 on the host.
"""
import math
import os

import numpy as np
import pytest

from oracle import dns_oracle as do

pytestmark = pytest.mark.gpu

K0, SEED, RE, CFL, UPDATE, METHOD = 15.0, 4895, 1e5, 0.1, 100, "LS_IMEX_RK3"


@pytest.fixture(scope="module")
def ts(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from palinstrophy_gb300 import turbo_simulator
    return turbo_simulator


def _oracle_run(N, steps):
    """FP64 oracle from the identical initial arrays: (start, final state, NEXTDT log)."""
    from palinstrophy_gb300 import _lib as L
    om2, uc, st = L.pao_generate(N, K0, RE, SEED, "KM3")
    S = do.OracleState(N, om2, uc, st["visc"], CFL, dtype=np.float64, workers=os.cpu_count() or 1)
    cflm0 = do.init_dt(S)
    dt0 = S.dt
    log = []
    do.run(S, steps, METHOD, UPDATE, log=log)
    return {"om2": om2, "uc": uc, "visc": float(st["visc"]), "cflm0": cflm0, "dt0": dt0, "log": log,
            "steps": steps, "S": S}


@pytest.fixture(scope="module")
def run4096(ts):
    return _oracle_run(4096, 100)


@pytest.fixture(scope="module")
def run2048(ts):
    return _oracle_run(2048, 10)


def _gpu_replayed(ts, N, prec, ref, variant=None, check_nextdt=False):
    """GPU run from the oracle's start with the oracle's dt / cn sequence replayed."""
    F = ts.Field(N, prec, RE, CFL)
    if variant is not None:
        F.set_variant(*variant)
    F.set_state(ref["om2"], None, ref["uc"])
    F.set_scalar("visc", ref["visc"])
    F.step2a()
    c0 = F.compute_cflm()
    F.set_scalar("dt", ref["dt0"])
    F.set_scalar("cn", 1.0)
    F.set_scalar("cnm1", 0.0)
    log = ref["log"]
    marks = [row[0] for row in log]
    done, own = 0, None
    for i, m in enumerate(marks):
        F.step(METHOD, m - done, update=0)
        done = m
        if i == 0 and check_nextdt:
            cflm = F.next_dt(sync_host=True)
            sc = F.scalars()
            own = (cflm, sc["dt"], sc["cn"])
        F.set_scalar("dt", log[i][2])
        F.set_scalar("cn", log[i][3])
    assert done == ref["steps"]
    out = (F.om2(), F.fnm1(), c0, own, F.variant()["desc"])
    F.close()
    return out


def _check_fp64(ts, N, ref):
    om, fn, c0, own, desc = _gpu_replayed(ts, N, "fp64", ref, check_nextdt=True)
    assert abs(c0 - ref["cflm0"]) <= 1e-13 * ref["cflm0"]
    it1 = ref["log"][0]
    cflm, dt, cn = own
    assert abs(cflm - it1[4]) <= 1e-12 * it1[4]
    assert abs(dt - it1[2]) <= 1e-12 * it1[2]
    assert abs(cn - it1[3]) <= 1e-12
    err = do.rel_l2(ref["S"].om2, om)
    assert err <= 1e-12, (desc, err)
    assert do.rel_l2(ref["S"].fnm1, fn) <= 1e-10, desc
    return err


def _check_fp32_all_candidates(ts, N, ref):
    F = ts.Field(N, "fp32", RE, CFL)
    v = F.variant()
    F.close()
    pairs = [(r, v["col"]) for r in range(v["n_rows"])] + [(v["row"], c) for c in range(v["n_cols"]) if c != v["col"]]
    errs = {}
    for pair in pairs:
        om, _, _, _, desc = _gpu_replayed(ts, N, "fp32", ref, variant=pair)
        errs[desc] = do.rel_l2(ref["S"].om2, om)
    worst = max(errs.values())
    assert worst <= 1e-4, errs
    return errs


def test_headline_n4096_fp64_100_steps_vs_oracle(ts, run4096):
    """FP64 GPU path (the autotuned kernels at N=4096) against the FP64 oracle."""
    _check_fp64(ts, 4096, run4096)


def test_headline_n4096_fp32_100_steps_vs_oracle(ts, run4096):
    """FP32 form against the FP64 oracle, every compiled row / column candidate at
    N=4096 -- among them the TMA row tiles and the TMA column pass the bench runs."""
    errs = _check_fp32_all_candidates(ts, 4096, run4096)
    assert any("tma" in d.split("col[")[1] for d in errs), errs


def test_headline_n4096_fp32_own_dt_vs_oracle(ts, run4096):
    """The bench's own path: FP32 form computing its own dt (FP64 CFL reductions)
    with the run_dns cadence, against the oracle's run; the NEXTDT values agree to
    FP32 accuracy and the field to 1e-4."""
    ref = run4096
    F = ts.Field(4096, "fp32", RE, CFL)
    F.set_state(ref["om2"], None, ref["uc"])
    F.set_scalar("visc", ref["visc"])
    F.step2a()
    F.set_scalar("dt", CFL / (F.compute_cflm() * math.pi))
    F.set_scalar("cn", 1.0)
    F.set_scalar("cnm1", 0.0)
    F.step(METHOD, 100, update=UPDATE, final_update=True)
    sc = F.scalars()
    assert abs(sc["dt"] - ref["S"].dt) <= 1e-5 * ref["S"].dt
    assert do.rel_l2(ref["S"].om2, F.om2()) <= 1e-4
    F.close()


def test_n2048_fp64_10_steps_vs_oracle(ts, run2048):
    _check_fp64(ts, 2048, run2048)


def test_n2048_fp32_10_steps_vs_oracle(ts, run2048):
    errs = _check_fp32_all_candidates(ts, 2048, run2048)
    assert any("tma" in d for d in errs), errs


@pytest.fixture(scope="module")
def run8192(ts):
    from palinstrophy_gb300 import _lib as L
    if not L.supported(8192, "fp32"):
        pytest.skip("fp32 is not compiled for N=8192")
    return _oracle_run(8192, 3)


def test_n8192_fp32_3_steps_vs_oracle(ts, run8192):
    """The FP32 form at N=8192 against the FP64 oracle after 3 steps (NEXTDT
    after step 1 replayed), for every row candidate -- the three cluster-split
    row passes among them -- and every column candidate."""
    errs = _check_fp32_all_candidates(ts, 8192, run8192)
    assert max(errs.values()) <= 1e-5, errs
    rows = {d.split(" col[")[0] for d in errs}
    assert sum("cluster" in r for r in rows) == 3, rows
