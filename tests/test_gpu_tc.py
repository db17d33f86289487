"""Tensor-core (tcgen05, 3-term split-BF16) SO(3) transform vs the FP64 oracle (GPU).

Tolerance: relative error <= 1e-6 (||a - b||_2 / ||b||_2) against FP64, the
bound the split-BF16 path is built to; complex64 grids and coefficients.
"""
import numpy as np
import pytest

from conftest import rel_err, so3_coeffs

pytestmark = pytest.mark.gpu
TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _tc_roundtrip(gblib, torch, L, batch, F, grid, recursion="stable", flags=0):
    p = gblib.Plan(gblib.SO3_COMPLEX, L, batch, "tc_bf16x3", recursion, flags)
    s = torch.cuda.current_stream().cuda_stream
    c = torch.from_numpy(np.ascontiguousarray(F.astype(np.complex64))).cuda()
    g = torch.from_numpy(np.ascontiguousarray(grid.astype(np.complex64))).cuda()
    gout = torch.empty_like(g)
    cout = torch.empty_like(c)
    p.inverse(c.data_ptr(), gout.data_ptr(), s)
    p.forward(g.data_ptr(), cout.data_ptr(), s)
    p.check()
    return gout.cpu().numpy().astype(np.complex128), cout.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("L", [5, 16, 31])
def test_tc_matches_fp64_oracle(gblib, oracle, torch_cuda, L):
    N = 2 * (L + 1)
    F = so3_coeffs(L, seed=L, decay="pow")
    g_ref = oracle.so3_inverse_complex_grid(L, F)
    G_ref = oracle.so3_forward_complex(L, g_ref)
    g, G = _tc_roundtrip(gblib, torch_cuda, L, 1, F, g_ref, recursion="reference")
    assert rel_err(g.reshape(N, N, N), g_ref) < TOL
    assert rel_err(G, G_ref) < TOL


def test_tc_batch_and_columns(gblib, oracle, torch_cuda):
    """17 functions: two 128-column tiles, functions in both."""
    L, b = 9, 17
    N = 2 * (L + 1)
    Fs = np.stack([so3_coeffs(L, seed=40 + i, decay="pow") for i in range(b)])
    gs = np.stack([oracle.so3_inverse_complex_grid(L, Fs[i]) for i in range(b)])
    g, G = _tc_roundtrip(gblib, torch_cuda, L, b, Fs.ravel(), gs.ravel(), recursion="reference")
    g = g.reshape(b, N, N, N)
    G = G.reshape(b, -1)
    for i in range(b):
        assert rel_err(g[i], gs[i]) < TOL
        assert rel_err(G[i], Fs[i]) < TOL
