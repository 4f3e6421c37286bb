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


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("name", ["init_KM3_N64_s4895_k10", "init_KM3_N128_s4895_k15", "init_KM3_N256_s4895_k10",
                                  "init_PAO_N128_s4895_k15", "init_PAO_N64_s7_k12"])
def test_host_generator_is_the_reference_field(built_lib, name):
    """The product generator (C++ LCG and shells, NumPy float32 cos/sin/exp) gives
    the reference's own arrays bit for bit -- signs of zero modes included -- and
    its printed Energy / WiWi and final seed."""
    d = golden(name + ".npz")
    om2, uc, st = L.pao_generate(int(d["N"]), float(d["K0"]), float(d["Re"]), int(d["seed"]), str(d["spectrum"]))
    assert np.array_equal(_bits(om2), _bits(d["om2"]))
    assert np.array_equal(_bits(uc), _bits(d["uc_low"]))
    assert st["seed_out"] == int(d["seed_out"])
    assert abs(st["Energy"] - float(d["Energy"])) <= 1e-8 * abs(float(d["Energy"]))
    assert abs(st["WiWi"] - float(d["WiWi"])) <= 1e-7 * abs(float(d["WiWi"]))
    assert np.float32(st["visc"]) == d["visc"]


@pytest.mark.parametrize("N,K0,seed,spec", [(96, 12.0, 7, "KM3"), (160, 6.0, 11, "PAO"), (200, 20.0, 5010, "KM3")])
def test_host_generator_matches_oracle_restatement(built_lib, N, K0, seed, spec):
    """Sizes and seeds without a fixture: the product equals the oracle's scalar
    restatement of the reference generator bit for bit, moments exactly."""
    om2, uc, st = L.pao_generate(N, K0, 1e4, seed, spec)
    g = pg.generate(N, K0, 1e4, seed, spec)
    assert np.array_equal(_bits(om2), _bits(g["om2"]))
    assert np.array_equal(_bits(uc), _bits(g["uc_low"]))
    assert st["seed_out"] == g["seed_out"]
    assert st["Energy"] == g["Q2"] and st["WiWi"] == g["W2"]


def test_libm_generator_close(built_lib):
    """pal_pao_generate takes cos/sin/exp from the C library, which may differ
    from NumPy's float32 ufuncs in the last bit: a few ulp, seeds exact."""
    d = golden("init_PAO_N64_s7_k12.npz")
    om2, uc, st = L.pao_generate_libm(64, 12.0, 1e4, 7, "PAO")
    assert st["seed_out"] == int(d["seed_out"])
    scale = np.abs(d["uc_low"]).max()
    assert np.abs(uc - d["uc_low"]).max() <= 4e-7 * scale
    assert np.abs(om2 - d["om2"]).max() <= 4e-7 * np.abs(d["om2"]).max()
    assert abs(st["Energy"] - float(d["Energy"])) < 1e-6
    om2, uc, st = L.pao_generate_libm(128, 15.0, 1e4, 4895, "KM3")
    g = golden("init_KM3_N128_s4895_k15.npz")
    assert np.abs(uc - g["uc_low"]).max() <= 4e-7 * np.abs(g["uc_low"]).max()


def test_host_generator_rejects_bad_n(built_lib):
    buf = np.zeros(16, np.complex64)
    f = np.zeros(16, np.float32)
    assert built_lib.pal_pao_generate(30, 10.0, 1e4, 1, 0, L.ptr(buf), L.ptr(buf), None, None) == L.PAL_ERR_INVALID
    assert built_lib.pal_pao_draws(30, 1, L.ptr(f), None) == L.PAL_ERR_INVALID
    assert built_lib.pal_pao_build(64, 10.0, 1e4, 1, 0, None, L.ptr(f), L.ptr(f), L.ptr(buf), L.ptr(buf),
                                   None) == L.PAL_ERR_INVALID
    with pytest.raises(ValueError):
        L.pao_generate(30, 10.0, 1e4, 1)
