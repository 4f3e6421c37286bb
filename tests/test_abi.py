"""C-ABI checks that need no GPU: the library loads, exports every entry point
that include/palgpu.h declares, validates arguments before touching CUDA, and
its host-side initial-condition generator reproduces the oracle's."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from oracle import pao_generator as pg
from palinstrophy_gb300 import _lib as L


def test_exports_every_header_symbol(built_lib):
    names = L.header_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(built_lib, n), n
    assert set(L._SIGS) == set(names), "ctypes signature table out of sync with the header"


def test_supported_sizes(built_lib):
    for n in (32, 64, 128, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096):
        assert built_lib.pal_supported(n, L.PAL_FP32) == 1
        assert built_lib.pal_supported(n, L.PAL_FP64) == 1
    assert built_lib.pal_supported(8192, L.PAL_FP32) == 1
    assert built_lib.pal_supported(8192, L.PAL_FP64) == 0
    assert built_lib.pal_supported(100, L.PAL_FP32) == 0
    assert built_lib.pal_supported(64, 7) == 0


def test_create_rejects_bad_arguments_before_cuda(built_lib):
    h = L._H()
    assert built_lib.pal_create(100, L.PAL_FP32, 1e4, 0.5, ctypes.byref(h)) == L.PAL_ERR_INVALID
    assert "unsupported grid" in L.last_error()
    assert built_lib.pal_create(64, 3, 1e4, 0.5, ctypes.byref(h)) == L.PAL_ERR_INVALID
    assert built_lib.pal_create(64, L.PAL_FP32, -1.0, 0.5, ctypes.byref(h)) == L.PAL_ERR_INVALID
    assert built_lib.pal_create(64, L.PAL_FP32, 1e4, 0.5, None) == L.PAL_ERR_INVALID
    assert h.value is None


def test_null_handle_is_an_error_not_a_crash(built_lib):
    assert built_lib.pal_step(None, 0, 1, 0, 0) == L.PAL_ERR_INVALID
    assert built_lib.pal_step2b(None) == L.PAL_ERR_INVALID
    assert built_lib.pal_destroy(None) == L.PAL_OK
    with pytest.raises(ValueError):
        L.check(built_lib.pal_step3(None))


@pytest.mark.parametrize("N,K0,seed", [(64, 10.0, 4895), (128, 15.0, 4895), (96, 12.0, 7)])
def test_host_generator_km3_matches_oracle(built_lib, N, K0, seed):
    """KM3 modes are computed in double, but their normalisation uses the PAO
    energy, whose float32 exp/sin/cos come from libm here and from NumPy's own
    float32 kernels in the reference: values agree to a few ulp (relative 3e-7), most exactly."""
    om2, uc, st = L.pao_generate(N, K0, 1e4, seed, "KM3")
    g = pg.generate(N, K0, 1e4, seed, "KM3")
    fa, fb = uc.view(np.float32), g["uc_low"].view(np.float32)
    assert (np.abs(fa - fb) <= 3e-7 * np.abs(fb)).all()
    assert (fa == fb).mean() > 0.9
    assert np.abs(om2 - g["om2"]).max() <= 3e-7 * np.abs(g["om2"]).max()
    assert st["seed_out"] == g["seed_out"]
    assert abs(st["Energy"] - g["Q2"]) <= 1e-7 * g["Q2"]
    assert np.float32(st["visc"]) == g["visc"]


def test_host_generator_pao_close(built_lib):
    """PAO uses float32 exp/sin/cos; libm and NumPy may differ in the last bit."""
    d = golden("init_PAO_N64_s7_k12.npz")
    om2, uc, st = L.pao_generate(64, 12.0, 1e4, 7, "PAO")
    assert st["seed_out"] == int(d["seed_out"])
    scale = np.abs(d["uc_low"]).max()
    assert np.abs(uc - d["uc_low"]).max() <= 4e-7 * scale
    assert np.abs(om2 - d["om2"]).max() <= 4e-7 * np.abs(d["om2"]).max()
    assert abs(st["Energy"] - float(d["Energy"])) < 1e-6


def test_host_generator_rejects_bad_n(built_lib):
    buf = np.zeros(16, np.complex64)
    assert built_lib.pal_pao_generate(30, 10.0, 1e4, 1, 0, L.ptr(buf), L.ptr(buf), None, None) == L.PAL_ERR_INVALID
