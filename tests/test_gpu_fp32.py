"""FP32 form of the beta-sum (FFTSO3_PREC_FP32: FP32 table, FP32 FMA accumulation on the
CUDA cores, FP32 FFT) vs the FP64 oracle (GPU).  Tolerance: relative error <= 1e-6
(||a - b||_2 / ||b||_2); complex64 / float32 data."""
import numpy as np
import pytest

from conftest import rel_err, s2_coeffs, so3_coeffs

pytestmark = pytest.mark.gpu
TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _roundtrip(gblib, torch, kind, L, batch, F, grid):
    complex_ = kind in (gblib.SO3_COMPLEX, gblib.S2_COMPLEX)
    p = gblib.Plan(kind, L, batch, "fp32", "reference")
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


@pytest.mark.parametrize("L", [5, 16, 31, 47])
def test_fp32_so3_complex(gblib, oracle, torch_cuda, L):
    N = 2 * (L + 1)
    F = so3_coeffs(L, seed=1200 + L, decay="pow")
    g_ref = oracle.so3_inverse_complex_grid(L, F)
    G_ref = oracle.so3_forward_complex(L, g_ref)
    g, G = _roundtrip(gblib, torch_cuda, gblib.SO3_COMPLEX, L, 1, F, g_ref)
    assert rel_err(g.reshape(N, N, N), g_ref) < TOL
    assert rel_err(G, G_ref) < TOL


def test_fp32_so3_real_batch(gblib, oracle, torch_cuda):
    """Real kind, 17 functions (two column tiles)."""
    L, b = 9, 17
    Fs = np.stack([so3_coeffs(L, seed=1300 + i, complex_=False) for i in range(b)])
    gs = np.stack([oracle.so3_inverse_real_grid(L, Fs[i]) for i in range(b)])
    g, G = _roundtrip(gblib, torch_cuda, gblib.SO3_REAL, L, b, Fs.ravel(), gs.ravel())
    g = g.reshape(b, -1)
    G = G.reshape(b, -1)
    for i in range(b):
        assert rel_err(g[i], gs[i].ravel()) < TOL
        assert rel_err(G[i], Fs[i]) < TOL


@pytest.mark.parametrize("kind", ["complex", "real"])
def test_fp32_s2(gblib, oracle, torch_cuda, kind):
    L = 31
    N = 2 * (L + 1)
    if kind == "complex":
        F = s2_coeffs(L, seed=1400)
        g_ref = oracle.s2_inverse_complex_grid(L, F)
        k = gblib.S2_COMPLEX
    else:
        F = s2_coeffs(L, seed=1401, complex_=False)
        g_ref = oracle.s2_inverse_real_grid(L, F)
        k = gblib.S2_REAL
    g, G = _roundtrip(gblib, torch_cuda, k, L, 1, F, g_ref)
    assert rel_err(g.reshape(N, N), g_ref) < TOL
    assert rel_err(G, F) < TOL
