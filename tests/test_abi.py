"""The C ABI library: loads, exports every declared symbol, host-side entry
points and argument checks (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu

HEADER = os.path.join(ROOT, "include", "fftso3_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fftso3_\w+)\s*\(", src)))


def test_header_declares_the_api():
    names = declared_functions()
    for required in ["fftso3_plan_create", "fftso3_plan_destroy", "fftso3_forward", "fftso3_inverse",
                     "fftso3_forward_host", "fftso3_inverse_host", "fftso3_inverse_points",
                     "fftso3_last_error_string", "fftso3_weights", "fftso3_wigner_d"]:
        assert required in names


def test_library_exports_every_declared_symbol(gblib):
    L = gblib.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
        assert name in gblib.SIGNATURES, f"{name} missing from the ctypes binding"


def test_weights_match_oracle_bitwise(gblib, oracle):
    for l_max in [0, 1, 5, 16, 127, 255]:
        for kind, ref in [(gblib.SO3_COMPLEX, oracle.so3_weights), (gblib.S2_REAL, oracle.s2_weights)]:
            w = np.zeros(2 * (l_max + 1))
            gblib.check(gblib.lib().fftso3_weights(kind, l_max, w.ctypes.data_as(gblib._dp)))
            assert np.array_equal(w, ref(l_max))


def test_sizes(gblib):
    L = gblib.lib()
    assert L.fftso3_grid_elems(gblib.SO3_COMPLEX, 16) == 34 ** 3
    assert L.fftso3_coeff_elems(gblib.SO3_REAL, 16) == 17 * (4 * 17 * 17 - 1) // 3
    assert L.fftso3_grid_elems(gblib.S2_COMPLEX, 511) == 1024 ** 2
    assert L.fftso3_coeff_elems(gblib.S2_REAL, 511) == 512 ** 2
    assert L.fftso3_grid_elems(7, 3) == -1
    assert L.fftso3_coeff_elems(0, -1) == -1


@pytest.mark.parametrize("args,msg", [
    ((9, 5, 1, 0, 0, 0), "kind"),
    ((0, -1, 1, 0, 0, 0), "l_max"),
    ((0, 5, 0, 0, 0, 0), "batch"),
    ((0, 5, 1, 7, 0, 0), "precision"),
    ((0, 5, 1, 0, 3, 0), "recursion"),
    ((0, 5, 1, 0, 0, 0x10), "flag"),
    ((2, 600, 1, 1, 0, 0), "tensor-core"),
])
def test_plan_create_rejects_bad_arguments(gblib, args, msg):
    h = ctypes.c_void_p()
    rc = gblib.lib().fftso3_plan_create(ctypes.byref(h), *args[:5], ctypes.c_uint(args[5]))
    assert rc in (gblib.ERR_INVALID_ARG, gblib.ERR_UNSUPPORTED)
    assert msg in gblib.lib().fftso3_last_error_string().decode()
    assert not h.value


@pytest.mark.parametrize("lmax,flags,msg", [
    ([4, -1], 0, "l_max[1]"),
    ([], 0, "n_functions"),
    ([4], 0x80, "flag"),
])
def test_batch_create_rejects_bad_arguments(gblib, lmax, flags, msg):
    h = ctypes.c_void_p()
    arr = (ctypes.c_int * max(len(lmax), 1))(*lmax)
    rc = gblib.lib().fftso3_batch_create(ctypes.byref(h), gblib.SO3_REAL, arr, len(lmax), 0, 0,
                                         ctypes.c_uint(flags))
    assert rc == gblib.ERR_INVALID_ARG
    assert msg in gblib.lib().fftso3_last_error_string().decode()
    assert not h.value
    assert gblib.lib().fftso3_batch_grid_offset(None, 0) == -1
    assert gblib.lib().fftso3_batch_forward(None, None, None, None) == gblib.ERR_INVALID_ARG


def test_null_plan_is_rejected(gblib):
    L = gblib.lib()
    assert L.fftso3_forward(None, None, None, None) == gblib.ERR_INVALID_ARG
    assert L.fftso3_plan_destroy(None) == gblib.ERR_INVALID_ARG
    assert L.fftso3_weights(0, -2, None) == gblib.ERR_INVALID_ARG


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_is_reported(gblib):
    h = ctypes.c_void_p()
    rc = gblib.lib().fftso3_plan_create(ctypes.byref(h), 0, 5, 1, 0, 0, ctypes.c_uint(0))
    assert rc == gblib.ERR_NO_DEVICE
    with pytest.raises(gblib.FFTSO3Error):
        gblib.Plan(gblib.SO3_COMPLEX, 5)


def test_grid_fft_rejects_bad_arguments_without_device_work(gblib):
    """Argument checks of the stand-alone grid FFT come before any CUDA call."""
    L = gblib.lib()
    assert L.fftso3_grid_fft_workspace_bytes(100, 1) == 0
    assert L.fftso3_grid_fft_workspace_bytes(64, 0) == 0
    ws = ctypes.c_void_p(256)  # never dereferenced: every call below fails its checks first
    a, b = ctypes.c_void_p(4096), ctypes.c_void_p(8192)
    cases = [(100, 1, 1, a, b, ws, "N must be"), (64, 0, 1, a, b, ws, "number of grids"),
             (64, 1, 0, a, b, ws, "dir must be"), (64, 1, 1, a, a, ws, "in == out"),
             (64, 1, 1, a, b, ctypes.c_void_p(264), "256-byte aligned")]
    for N, nf, d, i, o, w, msg in cases:
        assert L.fftso3_grid_fft(N, nf, d, 0, i, o, w, None) == gblib.ERR_INVALID_ARG
        assert msg in L.fftso3_last_error_string().decode()
    assert L.fftso3_grid_fft_check(None, None) == gblib.ERR_INVALID_ARG
