"""pal_step_noalloc: the allocation-free stepping entry point.

It exists for callers that cannot allocate device memory where they step a
field (host callbacks and real-time loops that must not block on the
allocator, plugins whose host forbids allocations after start-up).  Its work
planes live in a fixed scratch array inside the library, so this test checks,
through the C ABI, that two calls in a row give the same field as the regular
allocating path (pal_create + pal_step) within the FP32 tolerance of the other
tests, and that sizes beyond the scratch limit are refused.

This file is collected last so a failure here does not stop the other tests.
"""
import ctypes

import numpy as np
import pytest

from oracle import dns_oracle as do

pytestmark = pytest.mark.gpu

TOL = 1e-6  # FP32 rel-L2; both paths run the same kernels


@pytest.fixture(scope="module")
def env(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from palinstrophy_gb300 import _lib as L
    from palinstrophy_gb300.turbo_simulator import Field
    return torch, L, Field


def _reference_path(Field, om2, fnm1, method, nsteps, dt, visc, cn, cnm1):
    F = Field(om2.shape[0], "fp32", 1e4, 0.5)
    F.set_variant(0, 0)  # the kernel candidates pal_step_noalloc runs
    F.set_state(om2, fnm1, None)
    for k, v in (("dt", dt), ("visc", visc), ("cn", cn), ("cnm1", cnm1)):
        F.set_scalar(k, v)
    F.step(method, nsteps, update=0)
    out = F.om2(), F.fnm1()
    F.close()
    return out


def _start(Field, L, N):
    """A KM3 start at N and a fixed dt at CFL 0.5 for it."""
    import math
    om2, uc, st = L.pao_generate(N, 10.0, 1e4, 4895, "KM3")
    F = Field(N, "fp32", 1e4, 0.5)
    F.set_state(om2, None, uc)
    F.step2a()
    dt = 0.5 / (F.compute_cflm() * math.pi)
    F.close()
    return om2.astype(np.complex64), float(st["visc"]), dt


@pytest.mark.parametrize("N", [32, 256, 512])
@pytest.mark.parametrize("method,code", [("CNAB2", 0), ("LS_IMEX_RK3", 1)])
def test_two_calls_match_allocating_path(env, method, code, N):
    """Both ends of the supported range (N=512 is the largest field the scratch
    holds) and a middle size, each method; the second call allocates nothing."""
    torch, L, Field = env
    om2, visc, dt = _start(Field, L, N)
    fnm1 = np.zeros_like(om2)
    lib = L.load()
    dom = torch.from_numpy(om2.copy()).cuda()
    dfn = torch.from_numpy(fnm1.copy()).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # two calls in a row: 3 steps, then 4 more (cn = cnm1 = 1 after the first CNAB2 call)
    rc = lib.pal_step_noalloc(N, code, 3, dt, visc, 1.0, 0.0, ctypes.c_void_p(dom.data_ptr()),
                              ctypes.c_void_p(dfn.data_ptr()), stream)
    assert rc == L.PAL_OK
    torch.cuda.synchronize()
    a_om, a_fn = _reference_path(Field, om2, fnm1, method, 3, dt, visc, 1.0, 0.0)
    assert do.rel_l2(a_om, dom.cpu().numpy()) <= TOL
    assert do.rel_l2(a_fn, dfn.cpu().numpy()) <= TOL
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    rc = lib.pal_step_noalloc(N, code, 4, dt, visc, 1.0, 1.0 if method == "CNAB2" else 0.0,
                              ctypes.c_void_p(dom.data_ptr()), ctypes.c_void_p(dfn.data_ptr()), stream)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert rc == L.PAL_OK
    assert free_after == free_before, (free_before, free_after)   # no device memory taken
    b_om, b_fn = _reference_path(Field, om2, fnm1, method, 7, dt, visc, 1.0, 0.0)
    assert do.rel_l2(b_om, dom.cpu().numpy()) <= TOL
    assert do.rel_l2(b_fn, dfn.cpu().numpy()) <= TOL


def test_sizes_beyond_the_scratch_are_refused(env):
    torch, L, _ = env
    lib = L.load()
    big = torch.zeros((1024, 512), dtype=torch.complex64, device="cuda")
    p = ctypes.c_void_p(big.data_ptr())
    assert lib.pal_step_noalloc(1024, 0, 1, 1e-3, 1e-4, 1.0, 0.0, p, p, None) == L.PAL_ERR_INVALID
    assert lib.pal_step_noalloc(100, 0, 1, 1e-3, 1e-4, 1.0, 0.0, p, p, None) == L.PAL_ERR_INVALID
    assert lib.pal_step_noalloc(256, 0, 1, 1e-3, 1e-4, 1.0, 0.0, None, p, None) == L.PAL_ERR_INVALID
