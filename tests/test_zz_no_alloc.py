"""The allocation-free forward transform (fftso3_forward_noalloc) against the
plan-based one (GPU).

fftso3_forward_noalloc exists for callers that cannot allocate device memory:
a host that owns all device memory and does not let libraries call
cudaMalloc, or a latency-critical loop where cudaMalloc/cudaFree would
synchronise the device.  Its intermediates live in a fixed file-scope device
array, so it only accepts l_max <= FFTSO3_NOALLOC_MAX_LMAX.  This file is
named to be collected last; it builds the library itself, so it also runs
alone in a fresh process.

Tolerance: 1e-12 relative (the FP64 parity bound used by the other tests);
both paths use the same tables and kernels, so the results agree far better.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err, so3_coeffs

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("L", [0, 5, 16, 31])
def test_noalloc_forward_matches_plan_forward_twice(gblib, torch_cuda, L):
    torch = torch_cuda
    N = 2 * (L + 1)
    F = so3_coeffs(L, seed=300 + L)
    plan = gblib.Plan(gblib.SO3_COMPLEX, L, 1, "fp64", "reference")
    s = torch.cuda.current_stream().cuda_stream
    c = torch.from_numpy(F).cuda()
    grid = torch.empty(N ** 3, dtype=torch.complex128, device="cuda")
    plan.inverse(c.data_ptr(), grid.data_ptr(), s)
    ref = torch.empty_like(c)
    plan.forward(grid.data_ptr(), ref.data_ptr(), s)
    lib = gblib.lib()
    outs = []
    for _ in range(2):  # two calls in a row share the scratch array
        out = torch.full_like(c, float("nan"))
        gblib.check(lib.fftso3_forward_noalloc(L, ctypes.c_void_p(grid.data_ptr()),
                                               ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(s)))
        outs.append(out)
    torch.cuda.synchronize()
    want = ref.cpu().numpy()
    for out in outs:
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_err(got, want) < TOL


@pytest.mark.parametrize("L", [5, 31])
def test_noalloc_forward_matches_oracle_twice(gblib, oracle, torch_cuda, L):
    """Independent data and an independent check: the grid is the oracle's FP64 synthesis of seeded
    coefficients and the expected coefficients are the oracle's forward of that grid (the reference
    algorithm restated on the CPU), not the plan path's."""
    torch = torch_cuda
    F = so3_coeffs(L, seed=700 + L)
    g_ref = oracle.so3_inverse_complex_grid(L, F)
    want = oracle.so3_forward_complex(L, g_ref)
    s = torch.cuda.current_stream().cuda_stream
    grid = torch.from_numpy(np.ascontiguousarray(g_ref).ravel()).cuda()
    lib = gblib.lib()
    for _ in range(2):
        out = torch.full((want.size,), float("nan"), dtype=torch.complex128, device="cuda")
        gblib.check(lib.fftso3_forward_noalloc(L, ctypes.c_void_p(grid.data_ptr()),
                                               ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(s)))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_err(got, want) < TOL


def test_noalloc_rejects_sizes_above_its_limit(gblib, torch_cuda):
    lib = gblib.lib()
    rc = lib.fftso3_forward_noalloc(32, ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == gblib.ERR_INVALID_ARG
    assert "FFTSO3_NOALLOC_MAX_LMAX" in lib.fftso3_last_error_string().decode()
    assert lib.fftso3_forward_noalloc(4, None, None, None) == gblib.ERR_INVALID_ARG
