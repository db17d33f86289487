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


def _plan_pair(gblib, torch, kind, L, batch, recursion, flags=0):
    return (gblib.Plan(kind, L, batch, "tc_bf16x3", recursion, flags),
            gblib.Plan(kind, L, batch, "fp64", recursion, 0))


@pytest.mark.parametrize("L", [15, 31, 47])
def test_tc_real_matches_oracle(gblib, oracle, torch_cuda, L):
    """FFTSO3_real on the tensor cores: real grids (float32), real-basis coefficients.

    l_max 15 and 47 (N = 32, 96) take the generic FFT, l_max 31 (N = 64) the
    tile FFT with real samples in and the real part out.
    """
    torch = torch_cuda
    N = 2 * (L + 1)
    Fr = so3_coeffs(L, seed=100 + L, complex_=False, decay="pow")
    g_ref = oracle.so3_inverse_real_grid(L, Fr)
    G_ref = oracle.so3_forward_real(L, g_ref)
    p = gblib.Plan(gblib.SO3_REAL, L, 1, "tc_bf16x3", "reference", 0)
    s = torch.cuda.current_stream().cuda_stream
    c = torch.from_numpy(Fr.astype(np.float32)).cuda()
    g = torch.from_numpy(np.ascontiguousarray(g_ref.astype(np.float32))).cuda()
    gout = torch.empty_like(g)
    cout = torch.empty_like(c)
    p.inverse(c.data_ptr(), gout.data_ptr(), s)
    p.forward(g.data_ptr(), cout.data_ptr(), s)
    p.check()
    assert rel_err(gout.cpu().numpy().astype(np.float64).reshape(N, N, N), g_ref) < TOL
    assert rel_err(cout.cpu().numpy().astype(np.float64), G_ref) < TOL
    assert rel_err(cout.cpu().numpy().astype(np.float64), Fr) < TOL


def test_tc_real_refined_batch(gblib, oracle, torch_cuda):
    """Real kind, batch 3, with the residual refinement step on."""
    torch = torch_cuda
    L, b = 31, 3
    Frs = np.stack([so3_coeffs(L, seed=200 + i, complex_=False, decay="pow") for i in range(b)])
    gs = np.stack([oracle.so3_inverse_real_grid(L, Frs[i]) for i in range(b)])
    p = gblib.Plan(gblib.SO3_REAL, L, b, "tc_bf16x3", "reference", gblib.FLAG_REFINE)
    s = torch.cuda.current_stream().cuda_stream
    g = torch.from_numpy(np.ascontiguousarray(gs.astype(np.float32))).cuda()
    cout = torch.empty(Frs.shape, dtype=torch.float32, device="cuda")
    p.forward(g.data_ptr(), cout.data_ptr(), s)
    p.check()
    G = cout.cpu().numpy().astype(np.float64)
    for i in range(b):
        assert rel_err(G[i], Frs[i]) < TOL


def test_tc_generic_fft_lmax96(gblib, torch_cuda):
    """l_max = 96 (N = 194, not a power of two: mixed-radix FFT + transposes)
    against the FP64 plan, stable recursion, batch 2."""
    torch = torch_cuda
    L, b = 96, 2
    C = (L + 1) * (4 * (L + 1) ** 2 - 1) // 3
    F = np.concatenate([so3_coeffs(L, seed=300 + i, decay="pow") for i in range(b)])
    ptc, p64 = _plan_pair(gblib, torch, gblib.SO3_COMPLEX, L, b, "stable")
    s = torch.cuda.current_stream().cuda_stream
    c64 = torch.from_numpy(F).cuda()
    g64 = torch.empty(b * (2 * L + 2) ** 3, dtype=torch.complex128, device="cuda")
    p64.inverse(c64.data_ptr(), g64.data_ptr(), s)
    c32 = c64.to(torch.complex64)
    g32 = torch.empty(g64.shape, dtype=torch.complex64, device="cuda")
    ptc.inverse(c32.data_ptr(), g32.data_ptr(), s)
    ptc.check()
    assert rel_err(g32.cpu().numpy().astype(np.complex128), g64.cpu().numpy()) < TOL
    F32 = torch.empty(b * C, dtype=torch.complex64, device="cuda")
    ptc.forward(g64.to(torch.complex64).data_ptr(), F32.data_ptr(), s)
    ptc.check()
    assert rel_err(F32.cpu().numpy().astype(np.complex128), F) < TOL


@pytest.mark.parametrize("L", [63, 127])
def test_tc_tile_fft_sizes(gblib, torch_cuda, L):
    """Tile FFT at N = 128 and 256 (R = 4, 8) against the FP64 plan, stable recursion."""
    torch = torch_cuda
    C = (L + 1) * (4 * (L + 1) ** 2 - 1) // 3
    F = so3_coeffs(L, seed=1500 + L, decay="pow")
    ptc, p64 = _plan_pair(gblib, torch, gblib.SO3_COMPLEX, L, 1, "stable")
    s = torch.cuda.current_stream().cuda_stream
    c64 = torch.from_numpy(F).cuda()
    g64 = torch.empty((2 * L + 2) ** 3, dtype=torch.complex128, device="cuda")
    p64.inverse(c64.data_ptr(), g64.data_ptr(), s)
    g32 = torch.empty(g64.shape, dtype=torch.complex64, device="cuda")
    ptc.inverse(c64.to(torch.complex64).data_ptr(), g32.data_ptr(), s)
    F32 = torch.empty(C, dtype=torch.complex64, device="cuda")
    ptc.forward(g64.to(torch.complex64).data_ptr(), F32.data_ptr(), s)
    ptc.check()
    assert rel_err(g32.cpu().numpy().astype(np.complex128), g64.cpu().numpy()) < TOL
    assert rel_err(F32.cpu().numpy().astype(np.complex128), F) < TOL


def test_host_calls_pinned_equal_pageable(gblib, torch_cuda):
    """The host-buffer calls read/write pinned buffers in place and stage pageable ones;
    both give bit-identical results (tensor-core plan, batch 2)."""
    torch = torch_cuda
    L, b = 16, 2
    N = 2 * (L + 1)
    C = (L + 1) * (4 * (L + 1) ** 2 - 1) // 3
    p = gblib.Plan(gblib.SO3_COMPLEX, L, b, "tc_bf16x3", "reference")
    F = np.concatenate([so3_coeffs(L, seed=2100 + i) for i in range(b)]).astype(np.complex64)
    g_pageable = np.empty(b * N ** 3, dtype=np.complex64)
    p.inverse_host(F.ctypes.data, g_pageable.ctypes.data)
    c_pageable = np.empty_like(F)
    p.forward_host(g_pageable.ctypes.data, c_pageable.ctypes.data)
    Fp = torch.from_numpy(F).pin_memory()
    gp = torch.empty(b * N ** 3, dtype=torch.complex64).pin_memory()
    cp = torch.empty(b * C, dtype=torch.complex64).pin_memory()
    p.inverse_host(Fp.data_ptr(), gp.data_ptr())
    p.forward_host(gp.data_ptr(), cp.data_ptr())
    assert np.array_equal(gp.numpy(), g_pageable)
    assert np.array_equal(cp.numpy(), c_pageable)
    assert rel_err(cp.numpy().astype(np.complex128), F.astype(np.complex128)) < TOL


@pytest.mark.parametrize("kind,L,b", [("complex", 31, 3), ("real", 31, 2), ("complex", 63, 2),
                                      ("real", 127, 1), ("complex", 255, 1), ("real", 255, 1)])
def test_fused_fft_bitwise_equals_two_pass(gblib, torch_cuda, monkeypatch, kind, L, b):
    """The one-launch FFT (both passes through the L2 ring of beta-slice chunks) gives
    bit-identical grids and coefficients to the two-launch FFT through a full work grid
    (FFTSO3_TWO_PASS_FFT=1), for complex and real grids, N = 64 .. 512."""
    torch = torch_cuda
    N = 2 * (L + 1)
    k = gblib.SO3_COMPLEX if kind == "complex" else gblib.SO3_REAL
    C = (L + 1) * (4 * (L + 1) ** 2 - 1) // 3
    dt = torch.complex64 if kind == "complex" else torch.float32
    gen = torch.Generator(device="cuda").manual_seed(L + b)
    grid = torch.randn(b * N ** 3, dtype=dt, device="cuda", generator=gen)
    coef = torch.randn(b * C, dtype=dt, device="cuda", generator=gen)
    s = torch.cuda.current_stream().cuda_stream
    out = []
    for two_pass in ("0", "1"):
        monkeypatch.setenv("FFTSO3_TWO_PASS_FFT", two_pass)
        p = gblib.Plan(k, L, b, "tc_bf16x3", "stable")
        g = torch.empty_like(grid)
        c = torch.empty_like(coef)
        p.inverse(coef.data_ptr(), g.data_ptr(), s)
        p.forward(grid.data_ptr(), c.data_ptr(), s)
        p.check()
        out.append((g.cpu(), c.cpu()))
        del p
    assert torch.equal(out[0][0], out[1][0])
    assert torch.equal(out[0][1], out[1][1])
    assert torch.isfinite(out[0][1]).all()


@pytest.mark.parametrize("kind,L,b,cl", [("so3", 31, 40, "2"), ("so3", 63, 64, "4"), ("s2", 127, 100, "2"),
                                         ("s2", 255, 130, "4")])
def test_gemm_clusters_bitwise_equal_single_cta(gblib, torch_cuda, monkeypatch, kind, L, b, cl):
    """Clusters of 2 or 4 CTAs sharing each table tile by TMA multicast (FFTSO3_GEMM_CLUSTER) give
    bit-identical results to one CTA per item (=1): the same products in the same order.  Batches
    whose column tiles do not fill the last cluster block (40 SO(3) functions = 3 tiles in blocks of 2,
    130 S^2 signals = 5 tiles in blocks of 4) run empty tiles."""
    torch = torch_cuda
    k = gblib.SO3_COMPLEX if kind == "so3" else gblib.S2_COMPLEX
    N = 2 * (L + 1)
    G = b * (N ** 3 if kind == "so3" else N ** 2)
    C = b * ((L + 1) * (4 * (L + 1) ** 2 - 1) // 3 if kind == "so3" else (L + 1) ** 2)
    gen = torch.Generator(device="cuda").manual_seed(L + b)
    grid = torch.randn(G, dtype=torch.complex64, device="cuda", generator=gen)
    coef = torch.randn(C, dtype=torch.complex64, device="cuda", generator=gen)
    s = torch.cuda.current_stream().cuda_stream
    out = []
    for c in ("1", cl):
        monkeypatch.setenv("FFTSO3_GEMM_CLUSTER", c)
        p = gblib.Plan(k, L, b, "tc_bf16x3", "stable")
        g = torch.empty_like(grid)
        co = torch.empty_like(coef)
        p.inverse(coef.data_ptr(), g.data_ptr(), s)
        p.forward(grid.data_ptr(), co.data_ptr(), s)
        p.check()
        out.append((g.cpu(), co.cpu()))
        del p
    assert torch.equal(out[0][0], out[1][0])
    assert torch.equal(out[0][1], out[1][1])


def test_gemm_cluster_autotune_bitwise_equal(gblib, torch_cuda):
    """FFTSO3_FLAG_AUTOTUNE times GEMM clusters of 1, 2 and 4 CTAs on the plan's own buffers and keeps the fastest;
    whichever it keeps, the results equal the untuned plan's bit for bit (64 functions at l_max = 63: four column
    tiles, so all three cluster sizes are candidates), and a second tuned plan of the same shape reuses the
    choice."""
    torch = torch_cuda
    L, b = 63, 64
    N = 2 * (L + 1)
    C = b * ((L + 1) * (4 * (L + 1) ** 2 - 1) // 3)
    gen = torch.Generator(device="cuda").manual_seed(7)
    grid = torch.randn(b * N ** 3, dtype=torch.complex64, device="cuda", generator=gen)
    coef = torch.randn(C, dtype=torch.complex64, device="cuda", generator=gen)
    s = torch.cuda.current_stream().cuda_stream
    out = []
    for flags in (0, gblib.FLAG_AUTOTUNE, gblib.FLAG_AUTOTUNE):
        p = gblib.Plan(gblib.SO3_COMPLEX, L, b, "tc_bf16x3", "stable", flags)
        g = torch.empty_like(grid)
        co = torch.empty_like(coef)
        p.inverse(coef.data_ptr(), g.data_ptr(), s)
        p.forward(grid.data_ptr(), co.data_ptr(), s)
        p.check()
        out.append((g.cpu(), co.cpu()))
        del p
    for o in out[1:]:
        assert torch.equal(out[0][0], o[0])
        assert torch.equal(out[0][1], o[1])


@pytest.mark.parametrize("kind", ["complex", "real"])
def test_tc_round_trip_lmax255(gblib, torch_cuda, kind):
    """The headline size, l_max = 255 (512^3 grid, one-launch FFT at N = 512, clusters off at batch 1):
    forward(inverse(F)) returns F within the split-BF16 bound, relative L2 <= 1e-6, and per degree l the
    relative error stays <= 1e-5 (size-independent properties at full size; the FP64 comparison at this
    size is bench.py's accuracy line)."""
    torch = torch_cuda
    L = 255
    cplx = kind == "complex"
    F = so3_coeffs(L, seed=2551, complex_=cplx, decay="pow")
    k = gblib.SO3_COMPLEX if cplx else gblib.SO3_REAL
    p = gblib.Plan(k, L, 1, "tc_bf16x3", "stable")
    s = torch.cuda.current_stream().cuda_stream
    c = torch.from_numpy(F.astype(np.complex64 if cplx else np.float32)).cuda()
    g = torch.empty(512 ** 3, dtype=torch.complex64 if cplx else torch.float32, device="cuda")
    c2 = torch.empty_like(c)
    p.inverse(c.data_ptr(), g.data_ptr(), s)
    p.forward(g.data_ptr(), c2.data_ptr(), s)
    p.check()
    out = c2.cpu().numpy().astype(np.complex128 if cplx else np.float64)
    ref = F.astype(np.complex64 if cplx else np.float32).astype(np.complex128 if cplx else np.float64)
    assert rel_err(out, ref) < TOL
    from conftest import degrees_so3
    deg = degrees_so3(L)
    for l in (0, 1, 64, 128, 200, 255):
        sel = deg == l
        assert rel_err(out[sel], ref[sel]) < 1e-5


@pytest.mark.parametrize("L,kind", [(10, "complex"), (12, "real"), (28, "complex"), (36, "real"), (60, "complex"),
                                    (22, "complex")])
def test_tc_prime_factor_fft(gblib, torch_cuda, L, kind):
    """Generic-N grids N = 2(l_max + 1) whose largest factor is a prime p > 8 (p = 11, 13, 23, 29,
    37, 61): the first FFT stage is the symmetric prime DFT.  TC vs the FP64 plan on the same
    coefficients, relative L2 <= 1e-6 for the grids and the coefficients, batch 2."""
    torch = torch_cuda
    cplx = kind == "complex"
    k = gblib.SO3_COMPLEX if cplx else gblib.SO3_REAL
    N = 2 * (L + 1)
    F = so3_coeffs(L, seed=3000 + L, complex_=cplx, decay="pow")
    ptc = gblib.Plan(k, L, 2, "tc_bf16x3", "stable")
    p64 = gblib.Plan(k, L, 1, "fp64", "stable")
    s = torch.cuda.current_stream().cuda_stream
    F2 = np.concatenate([F, F])
    c64 = torch.from_numpy(F).cuda()
    g64 = torch.empty(N ** 3, dtype=torch.complex128 if cplx else torch.float64, device="cuda")
    p64.inverse(c64.data_ptr(), g64.data_ptr(), s)
    c32 = torch.from_numpy(F2.astype(np.complex64 if cplx else np.float32)).cuda()
    g32 = torch.empty(2 * N ** 3, dtype=torch.complex64 if cplx else torch.float32, device="cuda")
    ptc.inverse(c32.data_ptr(), g32.data_ptr(), s)
    gin = torch.cat([g64, g64]).to(torch.complex64 if cplx else torch.float32)
    F32 = torch.empty_like(c32)
    ptc.forward(gin.data_ptr(), F32.data_ptr(), s)
    ptc.check()
    gref = g64.cpu().numpy()
    gg = g32.cpu().numpy().astype(np.complex128 if cplx else np.float64)
    assert rel_err(gg[:N ** 3], gref) < TOL and rel_err(gg[N ** 3:], gref) < TOL
    FF = F32.cpu().numpy().astype(np.complex128 if cplx else np.float64)
    assert rel_err(FF[:F.size], F) < TOL and rel_err(FF[F.size:], F) < TOL
