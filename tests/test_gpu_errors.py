"""Error paths of the GPU kernels that need no fault to test.

The kernels that move their tiles with TMA bulk copies wait for them on an
mbarrier with a bounded number of polls; when the bound runs out they set a
flag in the device scalars, wait (again bounded) for their own copies before
using the tile, and the next host call that reads the scalars returns
PAL_ERR_TIMEOUT and clears the flag.  A test switch gives the first wait no
polls, so the report path runs while the copies still complete normally.
"""
import math

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


def _tma_field(ts, L, N, om2, uc, visc):
    F = ts.Field(N, "fp32", 1e5, 0.1)
    v = F.variant()
    rows, cols = [], []
    for r in range(v["n_rows"]):
        F.set_variant(r, 0)
        if "tma-in" in F.variant()["desc"].split("col[")[0]:
            rows.append(r)
    for c in range(v["n_cols"]):
        F.set_variant(0, c)
        if "tma" in F.variant()["desc"].split("col[")[1]:
            cols.append(c)
    assert rows and cols, "no TMA row / column candidate at this size"
    F.set_variant(rows[0], cols[0])
    F.set_state(om2, None, uc)
    F.set_scalar("visc", visc)
    F.step2a()
    F.set_scalar("dt", 0.1 / (F.compute_cflm() * math.pi))
    F.set_scalar("cn", 1.0)
    F.set_scalar("cnm1", 0.0)
    return F


@pytest.mark.parametrize("N", [1024, 4096])
def test_timed_out_wait_is_reported_and_cleared(ts, N):
    from palinstrophy_gb300 import _lib as L
    om2, uc, st = L.pao_generate(N, 15.0, 1e5, 4895, "KM3")
    A = _tma_field(ts, L, N, om2, uc, st["visc"])
    B = _tma_field(ts, L, N, om2, uc, st["visc"])
    A.step("LS_IMEX_RK3", 2, update=0)
    B.set_debug(L.PAL_DBG_SKIP_FIRST_WAIT, 1)
    B.step("LS_IMEX_RK3", 2, update=0)
    with pytest.raises(L.PalError) as err:
        B.scalars()
    assert err.value.code == L.PAL_ERR_TIMEOUT
    assert "timed out" in str(err.value)
    B.scalars()                                   # the flag was cleared by the report
    assert np.array_equal(A.om2(), B.om2())       # the kernels still waited for their copies
    B.set_debug(L.PAL_DBG_SKIP_FIRST_WAIT, 0)
    B.step("LS_IMEX_RK3", 1, update=0)
    B.scalars()                                   # normal waits: no report
    with pytest.raises(ValueError):
        B.set_debug(7, 1)
    A.close()
    B.close()


@pytest.mark.parametrize("form", ["cluster tma-in mc tma-out", "cluster tma-in dsmem tma-out", "cluster tma-in tma-out"])
def test_cluster_split_timed_out_wait(ts, form):
    """The cluster-split N=8192 row pass in each of its input forms: a first
    phase wait given no polls is reported once as PAL_ERR_TIMEOUT, both CTAs
    still wait for their copies and meet at every cluster barrier, and the
    field equals an undisturbed run."""
    from palinstrophy_gb300 import _lib as L
    N = 8192
    if not L.supported(N, "fp32"):
        pytest.skip("fp32 is not compiled for N=8192")
    om2, uc, st = L.pao_generate(N, 15.0, 1e5, 4895, "KM3")
    fields = []
    for _ in range(2):
        F = ts.Field(N, "fp32", 1e5, 0.1)
        v = F.variant()
        idx = None
        for r in range(v["n_rows"]):
            F.set_variant(r, 0)
            if F.variant()["desc"].split(" col[")[0].endswith(form + "]"):
                idx = r
        assert idx is not None, form
        F.set_variant(idx, 0)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", st["visc"])
        F.step2a()
        F.set_scalar("dt", 0.1 / (F.compute_cflm() * math.pi))
        F.set_scalar("cn", 1.0)
        F.set_scalar("cnm1", 0.0)
        fields.append(F)
    A, B = fields
    A.step("LS_IMEX_RK3", 1, update=0)
    B.set_debug(L.PAL_DBG_SKIP_FIRST_WAIT, 1)
    B.step("LS_IMEX_RK3", 1, update=0)
    with pytest.raises(L.PalError) as err:
        B.scalars()
    assert err.value.code == L.PAL_ERR_TIMEOUT
    B.scalars()
    assert np.array_equal(A.om2(), B.om2())
    A.close()
    B.close()
