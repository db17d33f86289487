"""Tensor-core (tcgen05, 3-term split-BF16) S^2 transforms vs the FP64 oracle (GPU).

The associated-Legendre beta-sum runs on the same persistent tensor-core GEMM
as SO(3), with one group per order m (pairs m and -m).  Tolerance: relative
error <= 1e-6 (||a - b||_2 / ||b||_2) against FP64; complex64 / float32 data.
"""
import numpy as np
import pytest

from conftest import rel_err, s2_coeffs

pytestmark = pytest.mark.gpu
TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _roundtrip(gblib, torch, kind, L, batch, F, grid, flags=0):
    complex_ = kind == gblib.S2_COMPLEX
    p = gblib.Plan(kind, L, batch, "tc_bf16x3", "reference", flags)
    dt = np.complex64 if complex_ else np.float32
    s = torch.cuda.current_stream().cuda_stream
    c = torch.from_numpy(np.ascontiguousarray(F.astype(dt))).cuda()
    g = torch.from_numpy(np.ascontiguousarray(grid.astype(dt))).cuda()
    gout = torch.empty_like(g)
    cout = torch.empty_like(c)
    p.inverse(c.data_ptr(), gout.data_ptr(), s)
    p.forward(g.data_ptr(), cout.data_ptr(), s)
    p.check()
    wide = np.complex128 if complex_ else np.float64
    return gout.cpu().numpy().astype(wide), cout.cpu().numpy().astype(wide)


@pytest.mark.parametrize("L", [0, 5, 15, 31, 40, 63])
def test_s2_tc_complex(gblib, oracle, torch_cuda, L):
    """l_max 31 and 63 (N = 64, 128) take the tiled register FFT; the others the generic FFT."""
    N = 2 * (L + 1)
    F = s2_coeffs(L, seed=700 + L)
    g_ref = oracle.s2_inverse_complex_grid(L, F)
    G_ref = oracle.s2_forward_complex(L, g_ref)
    g, G = _roundtrip(gblib, torch_cuda, gblib.S2_COMPLEX, L, 1, F, g_ref)
    assert rel_err(g.reshape(N, N), g_ref) < TOL
    assert rel_err(G, G_ref) < TOL
    assert rel_err(G, F) < TOL


@pytest.mark.parametrize("L", [15, 31, 40])
def test_s2_tc_real(gblib, oracle, torch_cuda, L):
    N = 2 * (L + 1)
    F = s2_coeffs(L, seed=800 + L, complex_=False)
    g_ref = oracle.s2_inverse_real_grid(L, F)
    G_ref = oracle.s2_forward_real(L, g_ref)
    g, G = _roundtrip(gblib, torch_cuda, gblib.S2_REAL, L, 1, F, g_ref)
    assert rel_err(g.reshape(N, N), g_ref) < TOL
    assert rel_err(G, G_ref) < TOL


def test_s2_tc_batch_columns(gblib, oracle, torch_cuda):
    """33 functions: two 32-function column tiles of the S^2 GEMM, the second nearly empty."""
    L, b = 20, 33
    N = 2 * (L + 1)
    Fs = np.stack([s2_coeffs(L, seed=900 + i) for i in range(b)])
    gs = np.stack([oracle.s2_inverse_complex_grid(L, Fs[i]) for i in range(b)])
    g, G = _roundtrip(gblib, torch_cuda, gblib.S2_COMPLEX, L, b, Fs.ravel(), gs.ravel())
    g = g.reshape(b, N, N)
    G = G.reshape(b, -1)
    for i in range(b):
        assert rel_err(g[i], gs[i]) < TOL
        assert rel_err(G[i], Fs[i]) < TOL


def test_s2_tc_real_refined(gblib, oracle, torch_cuda):
    L = 63
    F = s2_coeffs(L, seed=950, complex_=False)
    g_ref = oracle.s2_inverse_real_grid(L, F)
    _, G = _roundtrip(gblib, torch_cuda, gblib.S2_REAL, L, 1, F, g_ref, flags=gblib.FLAG_REFINE)
    assert rel_err(G, F) < TOL


def test_s2_tc_lmax511_against_fp64_plan(gblib, torch_cuda):
    """N = 1024 (tile FFT with R = 32), real signals, batch 3, against the FP64 plan run on
    the same FP32-rounded samples and coefficients (the error of the transform itself; at
    l_max = 511 it is 7e-7 .. 9e-7, of which the FP32 FFT alone gives about 5e-7)."""
    torch = torch_cuda
    L, b = 511, 3
    F = np.concatenate([s2_coeffs(L, seed=1600 + i, complex_=False) for i in range(b)])
    s = torch.cuda.current_stream().cuda_stream
    p64 = gblib.Plan(gblib.S2_REAL, L, b, "fp64", "reference")
    ptc = gblib.Plan(gblib.S2_REAL, L, b, "tc_bf16x3", "reference")
    c32 = torch.from_numpy(F).cuda().float()
    c64 = c32.double()
    g64 = torch.empty(b * (2 * L + 2) ** 2, dtype=torch.float64, device="cuda")
    p64.inverse(c64.data_ptr(), g64.data_ptr(), s)
    g32 = torch.empty(g64.shape, dtype=torch.float32, device="cuda")
    ptc.inverse(c32.data_ptr(), g32.data_ptr(), s)
    gin = g64.float()
    F64 = torch.empty(F.shape, dtype=torch.float64, device="cuda")
    p64.forward(gin.double().data_ptr(), F64.data_ptr(), s)
    F32 = torch.empty(F.shape, dtype=torch.float32, device="cuda")
    ptc.forward(gin.data_ptr(), F32.data_ptr(), s)
    ptc.check()
    assert rel_err(g32.cpu().numpy().astype(np.float64), g64.cpu().numpy()) < TOL
    assert rel_err(F32.cpu().numpy().astype(np.float64), F64.cpu().numpy()) < TOL
