"""Batched ensembles on the GPU: every member must evolve exactly as the same
field stepped alone (same kernels, same per-member adaptive dt), with and
without CUDA-graph replay, and match the CPU oracle."""
import math

import numpy as np
import pytest

from oracle import dns_oracle as do

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ts(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from palinstrophy_gb300 import turbo_simulator
    return turbo_simulator


def _member_init(N, seed):
    from palinstrophy_gb300 import _lib as L
    return L.pao_generate(N, 8.0, 1e4, seed, "KM3")


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("method", ["CNAB2", "LS_IMEX_RK3"])
def test_members_equal_single_fields(ts, prec, method):
    Ns = [64, 128, 64, 32, 128]
    seeds = [3, 5, 7, 11, 13]
    E = ts.Ensemble(Ns, prec, 1e4, 0.5)
    for m, (n, sd) in enumerate(zip(Ns, seeds)):
        om2, uc, st = _member_init(n, sd)
        E.set_member(m, om2, None, uc)
        E.set_scalar(m, "visc", st["visc"])
    E.set_scalar(-1, "cflnum", 0.5)
    E.init_dt()
    E.step(method, 12, update=4, graph=True)
    E.step(method, 12, update=4, graph=True)  # replays the cached graph
    E.synchronize()
    dts = []
    for m, (n, sd) in enumerate(zip(Ns, seeds)):
        om2, uc, st = _member_init(n, sd)
        F = ts.Field(n, prec, 1e4, 0.5)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        F.step2a()
        F.set_scalar("dt", 0.5 / (F.compute_cflm() * math.pi))
        F.set_scalar("cn", 1.0)
        F.set_scalar("cnm1", 0.0)
        F.set_scalar("it", 0)
        F.step(method, 24, update=4)
        assert np.array_equal(F.om2(), E.om2(m)), m
        se, sf = E.scalars(m), F.scalars()
        assert se["dt"] == sf["dt"] and se["it"] == 24
        assert abs(se["t"] - sf["t"]) <= 1e-15 * sf["t"]
        dts.append(se["dt"])
        F.close()
    assert len(set(dts)) > 1  # per-member adaptive dt
    E.close()


def test_graph_replay_equals_direct_launches(ts):
    Ns = [128, 64]
    outs = []
    for graph in (True, False):
        E = ts.Ensemble(Ns, "fp32", 1e4, 0.5)
        for m, n in enumerate(Ns):
            om2, uc, st = _member_init(n, 21 + m)
            E.set_member(m, om2, None, uc)
            E.set_scalar(m, "visc", st["visc"])
        E.init_dt()
        for _ in range(3):
            E.step("CNAB2", 10, update=5, graph=graph)
        outs.append([E.om2(m) for m in range(len(Ns))])
        E.close()
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_member_matches_oracle(ts):
    from oracle import pao_generator as pg
    g = pg.generate(64, 10.0, 1e4, 4895, "KM3")
    E = ts.Ensemble([64, 128], "fp64", 1e4, 0.75)
    E.set_member(0, g["om2"], None, g["uc_low"])
    E.set_scalar(0, "visc", float(g["visc"]))
    om2b, ucb, stb = _member_init(128, 9)
    E.set_member(1, om2b, None, ucb)
    E.init_dt()
    E.step("CNAB2", 30, update=10)
    S = do.OracleState(64, g["om2"], g["uc_low"], g["visc"], 0.75)
    do.init_dt(S)
    do.run(S, 30, "CNAB2", update=10)
    # the oracle also updates at it == 30 (== STEPS); the ensemble call ends at 30 with
    # update 10 -> the same NEXTDT points
    assert do.rel_l2(S.om2, E.om2(0)) <= 1e-12
    assert abs(E.scalars(0)["dt"] - S.dt) <= 1e-13 * S.dt
    E.close()


def test_bad_member_sizes_rejected(ts):
    from palinstrophy_gb300 import _lib as L
    with pytest.raises(L.PalError):
        ts.Ensemble([64, 100], "fp32")


def test_sharded_members_equal_the_whole_ensemble(ts):
    """Members stepped as two rank shards (run one after the other here) give the
    same fields and scalars, bit for bit, as the same members in one ensemble."""
    import numpy as np
    from palinstrophy_gb300.ensemble_shards import gather_rows, run_ensemble_shard
    Ns = [32, 64, 32, 64, 32]
    seeds = [11, 12, 13, 14, 15]
    whole = run_ensemble_shard(Ns, seeds, 0, 1, nsteps=20, update=1, return_fields=True)
    parts = []
    for r in range(2):
        parts.extend(run_ensemble_shard(Ns, seeds, r, 2, nsteps=20, update=1, return_fields=True))
    parts = gather_rows(parts)  # no process group: rows as they are
    assert [p["member"] for p in parts] == list(range(len(Ns)))
    for a, b in zip(whole, parts):
        for k in ("t", "dt", "cn", "cflm", "it"):
            assert a[k] == b[k], (a["member"], k)
        assert np.array_equal(a["om2"], b["om2"])


def test_batched_autotune(ts):
    """Groups re-tuned on their batched shape still give the single-field results
    to rounding; tuning after a member is set is refused."""
    import numpy as np
    from palinstrophy_gb300 import _lib as L
    Ns = [64] * 4 + [128] * 3
    E = ts.Ensemble(Ns, "fp32", 1e4, 0.5)
    E.autotune()
    assert E.variant(64).startswith("row[") and E.variant(128).startswith("row[")
    inits = []
    for m, n in enumerate(Ns):
        om2, uc, st = L.pao_generate(n, 10.0, 1e4, m + 1, "KM3")
        inits.append((om2, uc, st))
        E.set_member(m, om2, None, uc)
        E.set_scalar(m, "visc", st["visc"])
    with pytest.raises(ts.L.PalError if hasattr(ts, "L") else Exception):
        E.autotune()
    E.init_dt()
    E.step("CNAB2", 10, update=1)
    for m in (0, 5):
        om2, uc, st = inits[m]
        F = ts.Field(Ns[m], "fp32", 1e4, 0.5)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        F.step2a()
        F.set_scalar("dt", 0.5 / (F.compute_cflm() * np.pi))
        F.step("CNAB2", 10, update=1)
        a, b = E.om2(m).astype(np.complex128), F.om2().astype(np.complex128)
        assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 2e-6
        F.close()
    E.close()


def test_members_with_bulk_tensor_row_loads(ts):
    """Members of 1024 and 2048 (sizes whose tuned row kernels load and store
    their tiles with TMA bulk tensor copies through per-group descriptors with
    a member dimension) step exactly like single fields."""
    Ns = [1024, 2048, 1024]
    seeds = [2, 4, 6]
    E = ts.Ensemble(Ns, "fp32", 1e4, 0.5)
    for m, (n, sd) in enumerate(zip(Ns, seeds)):
        om2, uc, st = _member_init(n, sd)
        E.set_member(m, om2, None, uc)
        E.set_scalar(m, "visc", st["visc"])
    E.init_dt()
    E.step("LS_IMEX_RK3", 6, update=3, graph=True)
    E.synchronize()
    for m, (n, sd) in enumerate(zip(Ns, seeds)):
        om2, uc, st = _member_init(n, sd)
        F = ts.Field(n, "fp32", 1e4, 0.5)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        F.step2a()
        F.set_scalar("dt", 0.5 / (F.compute_cflm() * math.pi))
        F.step("LS_IMEX_RK3", 6, update=3)
        assert F.variant()["desc"] == E.variant(n)
        assert np.array_equal(F.om2(), E.om2(m)), m
        assert np.array_equal(F.fnm1(), E.fnm1(m)), m
        F.close()
    E.close()


def _force(F, desc):
    """Select the row / column candidates named in an ensemble variant string."""
    want_row = desc.split("row[")[1].split("]")[0]
    want_col = desc.split("col[")[1].split("]")[0]
    v = F.variant()
    r = c = None
    for i in range(v["n_rows"]):
        F.set_variant(i, 0)
        if F.variant()["desc"].split("row[")[1].split("]")[0] == want_row:
            r = i
    for j in range(v["n_cols"]):
        F.set_variant(0, j)
        if F.variant()["desc"].split("col[")[1].split("]")[0] == want_col:
            c = j
    assert r is not None and c is not None, desc
    F.set_variant(r, c)


@pytest.mark.parametrize("method", ["CNAB2", "LS_IMEX_RK3"])
@pytest.mark.parametrize("graph", [True, False])
def test_fused_passes_over_three_sizes(ts, method, graph):
    """Members of N = 256, 384 and 512 advance with ONE launch per pass for all
    sizes (the groups' blocks laid out in one grid, each block running its
    size's kernel body); every member equals the same field stepped alone with
    the same kernel candidates, bit for bit, with its own adaptive dt."""
    Ns = [256, 384, 512, 256, 512, 384]
    seeds = [1, 2, 3, 4, 5, 6]
    E = ts.Ensemble(Ns, "fp32", 1e4, 0.5)
    for n in (256, 384, 512):
        assert E.variant(n).startswith("fused row[")
    for m, (n, sd) in enumerate(zip(Ns, seeds)):
        om2, uc, st = _member_init(n, sd)
        E.set_member(m, om2, None, uc)
        E.set_scalar(m, "visc", st["visc"])
    E.init_dt()
    E.step(method, 5, update=2, graph=graph)
    E.step(method, 5, update=2, graph=graph)
    E.synchronize()
    dts = []
    for m, (n, sd) in enumerate(zip(Ns, seeds)):
        om2, uc, st = _member_init(n, sd)
        F = ts.Field(n, "fp32", 1e4, 0.5)
        _force(F, E.variant(n))
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        F.step2a()
        F.set_scalar("dt", 0.5 / (F.compute_cflm() * math.pi))
        F.set_scalar("cn", 1.0)
        F.set_scalar("cnm1", 0.0)
        F.set_scalar("it", 0)
        F.step(method, 10, update=2)
        assert np.array_equal(F.om2(), E.om2(m)), m
        assert np.array_equal(F.fnm1(), E.fnm1(m)), m
        se, sf = E.scalars(m), F.scalars()
        assert se["dt"] == sf["dt"] and se["it"] == 10
        dts.append(se["dt"])
        F.close()
    assert len(set(dts)) > 1
    E.close()


def test_fused_passes_off_and_after_autotune(ts, monkeypatch):
    """PAL_ENSEMBLE_FUSED=0 and a batched re-tune both give per-size launches."""
    E = ts.Ensemble([256, 384], "fp32", 1e4, 0.5)
    E.autotune()
    assert not E.variant(256).startswith("fused")
    E.close()
    monkeypatch.setenv("PAL_ENSEMBLE_FUSED", "0")
    E = ts.Ensemble([256, 384], "fp32", 1e4, 0.5)
    assert not E.variant(384).startswith("fused")
    E.close()


def test_cluster_split_rows_with_members(ts):
    """Two N=8192 members run the autotuned cluster-split row pass (a tile per
    2-CTA cluster, one grid row per member, TMA descriptors with a member
    dimension) and step exactly like a single field on the same candidates."""
    from palinstrophy_gb300 import _lib as L
    if not L.supported(8192, "fp32"):
        pytest.skip("fp32 is not compiled for N=8192")
    Ns = [8192, 8192]
    E = ts.Ensemble(Ns, "fp32", 1e5, 0.1)
    assert "cluster" in E.variant(8192), E.variant(8192)
    inits = [L.pao_generate(8192, 15.0, 1e5, sd, "KM3") for sd in (3, 4)]
    for m, (om2, uc, st) in enumerate(inits):
        E.set_member(m, om2, None, uc)
        E.set_scalar(m, "visc", st["visc"])
    E.init_dt()
    E.step("LS_IMEX_RK3", 2, update=1, graph=True)
    E.synchronize()
    om2, uc, st = inits[1]
    F = ts.Field(8192, "fp32", 1e5, 0.1)
    F.set_state(om2, None, uc)
    F.set_scalar("visc", st["visc"])
    F.step2a()
    F.set_scalar("dt", 0.1 / (F.compute_cflm() * math.pi))
    F.step("LS_IMEX_RK3", 2, update=1)
    assert F.variant()["desc"] == E.variant(8192)
    assert np.array_equal(F.om2(), E.om2(1))
    assert E.scalars(1)["dt"] == F.scalars()["dt"]
    F.close()
    E.close()
