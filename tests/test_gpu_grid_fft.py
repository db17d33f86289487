"""The grid FFT stage on its own (fftso3_grid_fft, the one-launch transposing FFT)
against numpy's FFT (GPU).

dir = 1 maps grids g[f][k][j1][j2] to pencils P[f][p][q][k] = fft2 over (j1, j2);
dir = -1 maps pencils back with the same kernel e^{-2 pi i / N}.  FP32 arithmetic:
relative error (||a - b||_2 / ||b||_2) <= 1e-6 against numpy's FP64 FFT.  At
N = 512 the size-independent check is the double transform, which returns
N^2 g[k][-j1][-j2].
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _ws(torch, gblib, N, nf):
    n = gblib.grid_fft_workspace_bytes(N, nf)
    assert n > 0
    return torch.zeros(n + 256, dtype=torch.uint8, device="cuda")


def _aligned(t):
    p = t.data_ptr()
    return p + (-p) % 256


@pytest.mark.parametrize("N,nf", [(64, 3), (128, 2), (256, 1)])
@pytest.mark.parametrize("real", [False, True])
def test_grid_fft_matches_numpy(gblib, torch_cuda, N, nf, real):
    torch = torch_cuda
    rng = np.random.default_rng(N + nf + real)
    shape = (nf, N, N, N)
    g = rng.standard_normal(shape) + (0 if real else 1j * rng.standard_normal(shape))
    dt = np.float32 if real else np.complex64
    s = torch.cuda.current_stream().cuda_stream
    ws = _ws(torch, gblib, N, nf)
    gin = torch.from_numpy(np.ascontiguousarray(g.astype(dt))).cuda()
    pen = torch.empty(shape, dtype=torch.complex64, device="cuda")
    gblib.grid_fft(N, nf, 1, real, gin.data_ptr(), pen.data_ptr(), _aligned(ws), s)
    gblib.grid_fft_check(_aligned(ws), s)
    ref = np.fft.fft2(g.astype(dt).astype(np.complex128), axes=(2, 3)).transpose(0, 2, 3, 1)
    assert _rel(pen.cpu().numpy(), ref) < TOL
    # inverse direction: pencils -> grids with the same kernel; real grids come from Hermitian pencils
    # (P[-p][-q] = conj P[p][q]), here those of a real grid
    if real:
        P = np.fft.fft2(rng.standard_normal(shape), axes=(2, 3)).transpose(0, 2, 3, 1) / N
    else:
        P = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    pin = torch.from_numpy(np.ascontiguousarray(P.astype(np.complex64))).cuda()
    gout = torch.empty(shape, dtype=torch.float32 if real else torch.complex64, device="cuda")
    gblib.grid_fft(N, nf, -1, real, pin.data_ptr(), gout.data_ptr(), _aligned(ws), s)
    gblib.grid_fft_check(_aligned(ws), s)
    ref = np.fft.fft2(P.astype(np.complex64).astype(np.complex128).transpose(0, 3, 1, 2), axes=(2, 3))
    if real:
        ref = ref.real
    assert _rel(gout.cpu().numpy(), ref) < TOL


def test_grid_fft_double_transform_n512(gblib, torch_cuda):
    """N = 512, 2 grids: forward then inverse direction gives N^2 g[k][-j1][-j2]."""
    torch = torch_cuda
    N, nf = 512, 2
    gen = torch.Generator(device="cuda").manual_seed(7)
    g = torch.randn((nf, N, N, N), dtype=torch.complex64, device="cuda", generator=gen)
    pen = torch.empty_like(g)
    back = torch.empty_like(g)
    s = torch.cuda.current_stream().cuda_stream
    ws = _ws(torch, gblib, N, nf)
    gblib.grid_fft(N, nf, 1, False, g.data_ptr(), pen.data_ptr(), _aligned(ws), s)
    gblib.grid_fft(N, nf, -1, False, pen.data_ptr(), back.data_ptr(), _aligned(ws), s)
    gblib.grid_fft_check(_aligned(ws), s)
    idx = (-torch.arange(N, device="cuda")) % N
    expect = g[:, :, idx][:, :, :, idx] * (N * N)
    err = float(torch.linalg.vector_norm(back - expect) / torch.linalg.vector_norm(expect))
    assert err < 2 * TOL


def test_grid_fft_deterministic(gblib, torch_cuda):
    """Two calls on the same grid give bit-identical pencils (every tile is computed by one CTA
    with fixed arithmetic, whichever CTA claims it)."""
    torch = torch_cuda
    N, nf = 64, 1
    gen = torch.Generator(device="cuda").manual_seed(11)
    g = torch.randn((nf, N, N, N), dtype=torch.complex64, device="cuda", generator=gen)
    s = torch.cuda.current_stream().cuda_stream
    ws = _ws(torch, gblib, N, nf)
    pen1 = torch.empty_like(g)
    pen2 = torch.empty_like(g)
    gblib.grid_fft(N, nf, 1, False, g.data_ptr(), pen1.data_ptr(), _aligned(ws), s)
    gblib.grid_fft(N, nf, 1, False, g.data_ptr(), pen2.data_ptr(), _aligned(ws), s)
    gblib.grid_fft_check(_aligned(ws), s)
    assert torch.equal(pen1, pen2)


def test_grid_fft_rejects_bad_arguments(gblib, torch_cuda):
    torch = torch_cuda
    ws = _ws(torch, gblib, 64, 1)
    x = torch.zeros(64 ** 3, dtype=torch.complex64, device="cuda")
    y = torch.zeros_like(x)
    for args in [(100, 1, 1), (64, 0, 1), (64, 1, 0)]:
        with pytest.raises(gblib.FFTSO3Error):
            gblib.grid_fft(args[0], args[1], args[2], False, x.data_ptr(), y.data_ptr(), _aligned(ws), 0)
    with pytest.raises(gblib.FFTSO3Error):
        gblib.grid_fft(64, 1, 1, False, x.data_ptr(), x.data_ptr(), _aligned(ws), 0)
    with pytest.raises(gblib.FFTSO3Error):
        gblib.grid_fft(64, 1, 1, False, x.data_ptr(), y.data_ptr(), _aligned(ws) + 8, 0)
