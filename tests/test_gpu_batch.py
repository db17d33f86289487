"""Batches of uneven bandwidth (fftso3_batch_*) against per-function plans and the oracle (GPU).

Tolerances: the FP64 batch equals per-function FP64 plans bit for bit (same
kernels, same arithmetic per function); tensor-core results are within
1e-6 relative of the FP64 oracle, as for plans.
"""
import os

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


def _layout_ok(b, lmax, kind, gblib):
    """Bucket-major offsets, ascending l_max, caller order within a bucket, no overlap."""
    lib = gblib.lib()
    n = len(lmax)
    order = sorted(range(n), key=lambda i: (lmax[i], i))
    g = c = 0
    for i in order:
        assert b.grid_offset(i) == g and b.coeff_offset(i) == c
        g += lib.fftso3_grid_elems(kind, lmax[i])
        c += lib.fftso3_coeff_elems(kind, lmax[i])
    assert b.grid_elems == g and b.coeff_elems == c
    assert b.buckets == len(set(lmax))
    assert b.grid_offset(n + 1) == -1 and b.grid_offset(-1) == -1


def test_batch_real_tc_matches_oracle(gblib, oracle, torch_cuda):
    torch = torch_cuda
    lmax = [8, 12, 8, 20, 15, 12, 31, 9, 8]
    kind = gblib.SO3_REAL
    b = gblib.Batch(kind, lmax, "tc_bf16x3", "reference", gblib.FLAG_GRAPH)
    _layout_ok(b, lmax, kind, gblib)
    Fr = [so3_coeffs(L, seed=500 + i, complex_=False) for i, L in enumerate(lmax)]
    grids = [oracle.so3_inverse_real_grid(L, F) for L, F in zip(lmax, Fr)]
    gbuf = np.zeros(b.grid_elems, dtype=np.float32)
    cbuf = np.zeros(b.coeff_elems, dtype=np.float32)
    for i, L in enumerate(lmax):
        gbuf[b.grid_offset(i):b.grid_offset(i) + grids[i].size] = grids[i].ravel()
        cbuf[b.coeff_offset(i):b.coeff_offset(i) + Fr[i].size] = Fr[i]
    s = torch.cuda.current_stream().cuda_stream
    g = torch.from_numpy(gbuf).cuda()
    c = torch.from_numpy(cbuf).cuda()
    cout = torch.zeros_like(c)
    gout = torch.zeros_like(g)
    for _ in range(2):  # capture, then replay
        b.forward(g.data_ptr(), cout.data_ptr(), s)
        b.inverse(c.data_ptr(), gout.data_ptr(), s)
    b.check()
    co = cout.cpu().numpy().astype(np.float64)
    go = gout.cpu().numpy().astype(np.float64)
    for i, L in enumerate(lmax):
        F_i = co[b.coeff_offset(i):b.coeff_offset(i) + Fr[i].size]
        g_i = go[b.grid_offset(i):b.grid_offset(i) + grids[i].size]
        assert rel_err(F_i, Fr[i]) < TOL, (i, L)
        assert rel_err(g_i, grids[i].ravel()) < TOL, (i, L)


def test_batch_fp64_equals_plans(gblib, torch_cuda):
    """FP64 complex batch (graph and eager) equals one batch-1 plan per function, bit for bit."""
    torch = torch_cuda
    lmax = [5, 3, 5, 7, 3, 16]
    kind = gblib.SO3_COMPLEX
    s = torch.cuda.current_stream().cuda_stream
    Fs = [so3_coeffs(L, seed=600 + i) for i, L in enumerate(lmax)]
    outs = {}
    for flags in (0, gblib.FLAG_GRAPH):
        b = gblib.Batch(kind, lmax, "fp64", "reference", flags)
        _layout_ok(b, lmax, kind, gblib)
        cbuf = np.zeros(b.coeff_elems, dtype=np.complex128)
        for i in range(len(lmax)):
            cbuf[b.coeff_offset(i):b.coeff_offset(i) + Fs[i].size] = Fs[i]
        c = torch.from_numpy(cbuf).cuda()
        g = torch.zeros(b.grid_elems, dtype=torch.complex128, device="cuda")
        c2 = torch.zeros_like(c)
        b.inverse(c.data_ptr(), g.data_ptr(), s)
        b.forward(g.data_ptr(), c2.data_ptr(), s)
        # a second pointer pair forces a new capture in graph mode
        g2 = torch.zeros_like(g)
        b.inverse(c.data_ptr(), g2.data_ptr(), s)
        b.check()
        assert torch.equal(g, g2)
        outs[flags] = (b, g.cpu().numpy(), c2.cpu().numpy())
    b0, g0, c0 = outs[0]
    b1, g1, c1 = outs[gblib.FLAG_GRAPH]
    assert np.array_equal(g0, g1) and np.array_equal(c0, c1)
    for i, L in enumerate(lmax):
        p = gblib.Plan(kind, L, 1, "fp64", "reference")
        ci = torch.from_numpy(Fs[i]).cuda()
        gi = torch.zeros(p.grid_elems, dtype=torch.complex128, device="cuda")
        fi = torch.zeros_like(ci)
        p.inverse(ci.data_ptr(), gi.data_ptr(), s)
        p.forward(gi.data_ptr(), fi.data_ptr(), s)
        p.check()
        go, co = b0.grid_offset(i), b0.coeff_offset(i)
        assert np.array_equal(g0[go:go + p.grid_elems], gi.cpu().numpy())
        assert np.array_equal(c0[co:co + p.coeff_elems], fi.cpu().numpy())
        assert rel_err(c0[co:co + p.coeff_elems], Fs[i]) < 1e-12



def test_autotuned_plan_and_batch(gblib, oracle, torch_cuda):
    """FFTSO3_FLAG_AUTOTUNE changes only launch shapes: results stay within the tensor-core tolerance of the
    oracle, for a plan with a large prime factor in N (l_max = 60, N = 122 = 2 * 61) and for a batch."""
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    L = 60
    Fr = so3_coeffs(L, seed=1000, complex_=False)
    g_ref = oracle.so3_inverse_real_grid(L, Fr)
    for flags in (0, gblib.FLAG_AUTOTUNE):
        p = gblib.Plan(gblib.SO3_REAL, L, 2, "tc_bf16x3", "reference", flags)
        g = torch.from_numpy(np.concatenate([g_ref.ravel(), g_ref.ravel()]).astype(np.float32)).cuda()
        c = torch.empty(2 * Fr.size, dtype=torch.float32, device="cuda")
        p.forward(g.data_ptr(), c.data_ptr(), s)
        p.check()
        co = c.cpu().numpy().astype(np.float64)
        assert rel_err(co[:Fr.size], Fr) < TOL and rel_err(co[Fr.size:], Fr) < TOL
    lmax = [10, 33, 10, 21, 46, 33]
    b = gblib.Batch(gblib.SO3_REAL, lmax, "tc_bf16x3", "reference", gblib.FLAG_GRAPH | gblib.FLAG_AUTOTUNE)
    Fs = [so3_coeffs(l, seed=1100 + i, complex_=False) for i, l in enumerate(lmax)]
    cbuf = np.zeros(b.coeff_elems, dtype=np.float32)
    for i in range(len(lmax)):
        cbuf[b.coeff_offset(i):b.coeff_offset(i) + Fs[i].size] = Fs[i]
    c = torch.from_numpy(cbuf).cuda()
    g = torch.empty(b.grid_elems, dtype=torch.float32, device="cuda")
    c2 = torch.empty_like(c)
    b.inverse(c.data_ptr(), g.data_ptr(), s)
    b.forward(g.data_ptr(), c2.data_ptr(), s)
    b.check()
    assert 1 <= b.streams <= b.buckets
    co = c2.cpu().numpy().astype(np.float64)
    for i in range(len(lmax)):
        assert rel_err(co[b.coeff_offset(i):b.coeff_offset(i) + Fs[i].size], Fs[i]) < TOL


def _per_bucket_batch(gblib, *args):
    """A batch created with FFTSO3_BATCH_PHASES=0: per-bucket phases around the one fused GEMM launch."""
    old = os.environ.get("FFTSO3_BATCH_PHASES")
    os.environ["FFTSO3_BATCH_PHASES"] = "0"
    try:
        return gblib.Batch(*args)
    finally:
        if old is None:
            del os.environ["FFTSO3_BATCH_PHASES"]
        else:
            os.environ["FFTSO3_BATCH_PHASES"] = old


def test_fused_gemm_batch_equals_bucket_plans(gblib, torch_cuda):
    """The per-bucket form (FFTSO3_BATCH_PHASES=0) runs one GEMM launch over all buckets; every item is computed
    exactly as the bucket's own plan computes it, so the results are bit-identical to one plan per l_max
    (complex SO(3))."""
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    lmax = [12, 20, 12, 31, 20, 12]
    kind = gblib.SO3_COMPLEX
    b = _per_bucket_batch(gblib, kind, lmax, "tc_bf16x3", "reference", 0)
    assert b.streams >= 1
    Fs = [so3_coeffs(L, seed=1700 + i, decay="pow").astype(np.complex64) for i, L in enumerate(lmax)]
    cbuf = np.zeros(b.coeff_elems, dtype=np.complex64)
    for i in range(len(lmax)):
        cbuf[b.coeff_offset(i):b.coeff_offset(i) + Fs[i].size] = Fs[i]
    c = torch.from_numpy(cbuf).cuda()
    g = torch.empty(b.grid_elems, dtype=torch.complex64, device="cuda")
    c2 = torch.empty_like(c)
    b.inverse(c.data_ptr(), g.data_ptr(), s)
    b.forward(g.data_ptr(), c2.data_ptr(), s)
    b.check()
    for L in sorted(set(lmax)):
        idx = [i for i in range(len(lmax)) if lmax[i] == L]
        p = gblib.Plan(kind, L, len(idx), "tc_bf16x3", "reference")
        g0, c0 = b.grid_offset(idx[0]), b.coeff_offset(idx[0])
        n_g, n_c = len(idx) * p.grid_elems, len(idx) * p.coeff_elems
        gp = torch.empty(n_g, dtype=torch.complex64, device="cuda")
        cp = torch.empty(n_c, dtype=torch.complex64, device="cuda")
        p.inverse(c[c0:c0 + n_c].data_ptr(), gp.data_ptr(), s)
        p.forward(g[g0:g0 + n_g].data_ptr(), cp.data_ptr(), s)
        p.check()
        assert torch.equal(gp, g[g0:g0 + n_g])
        assert torch.equal(cp, c2[c0:c0 + n_c])


@pytest.mark.parametrize("kind", ["complex", "real"])
def test_three_launch_batch(gblib, oracle, torch_cuda, kind):
    """SO(3) tensor-core batches run each direction as three launches over all buckets (slice FFT, fused GEMM,
    coefficient conversion): the captured graphs hold three kernel nodes per direction, on one stream.  Results
    within 1e-6 of the oracle, and within 1e-6 (relative) of one plan per l_max -- the slice FFT rounds
    differently from the plans' FFTs.  l_max 60 (N = 122 = 2 * 61) takes the prime first stage; several slices
    share a CTA for the small l_max."""
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    cplx = kind == "complex"
    k = gblib.SO3_COMPLEX if cplx else gblib.SO3_REAL
    lmax = [8, 12, 8, 20, 15, 12, 31, 9, 8, 46, 60, 33, 60]
    b = gblib.Batch(k, lmax, "tc_bf16x3", "reference", gblib.FLAG_GRAPH)
    _layout_ok(b, lmax, k, gblib)
    Fs = [so3_coeffs(L, seed=1900 + i, complex_=cplx) for i, L in enumerate(lmax)]
    inv = oracle.so3_inverse_complex_grid if cplx else oracle.so3_inverse_real_grid
    grids = [inv(L, F) for L, F in zip(lmax, Fs)]
    npt, tt = (np.complex64, torch.complex64) if cplx else (np.float32, torch.float32)
    gbuf = np.zeros(b.grid_elems, dtype=npt)
    cbuf = np.zeros(b.coeff_elems, dtype=npt)
    for i in range(len(lmax)):
        gbuf[b.grid_offset(i):b.grid_offset(i) + grids[i].size] = grids[i].ravel()
        cbuf[b.coeff_offset(i):b.coeff_offset(i) + Fs[i].size] = Fs[i]
    g = torch.from_numpy(gbuf).cuda()
    c = torch.from_numpy(cbuf).cuda()
    cout = torch.zeros_like(c)
    gout = torch.zeros_like(g)
    for _ in range(2):  # capture, then replay
        b.forward(g.data_ptr(), cout.data_ptr(), s)
        b.inverse(c.data_ptr(), gout.data_ptr(), s)
    b.check()
    assert b.graph_kernels(0) == 3 and b.graph_kernels(1) == 3
    assert b.streams == 1
    wide = np.complex128 if cplx else np.float64
    co = cout.cpu().numpy().astype(wide)
    go = gout.cpu().numpy().astype(wide)
    for i, L in enumerate(lmax):
        F_i = co[b.coeff_offset(i):b.coeff_offset(i) + Fs[i].size]
        g_i = go[b.grid_offset(i):b.grid_offset(i) + grids[i].size]
        assert rel_err(F_i, Fs[i]) < TOL, (i, L)
        assert rel_err(g_i, grids[i].ravel()) < TOL, (i, L)
    for L in sorted(set(lmax)):
        idx = [i for i in range(len(lmax)) if lmax[i] == L]
        p = gblib.Plan(k, L, len(idx), "tc_bf16x3", "reference")
        g0, c0 = b.grid_offset(idx[0]), b.coeff_offset(idx[0])
        n_g, n_c = len(idx) * p.grid_elems, len(idx) * p.coeff_elems
        gp = torch.empty(n_g, dtype=tt, device="cuda")
        cp = torch.empty(n_c, dtype=tt, device="cuda")
        p.inverse(c[c0:c0 + n_c].data_ptr(), gp.data_ptr(), s)
        p.forward(g[g0:g0 + n_g].data_ptr(), cp.data_ptr(), s)
        p.check()
        assert rel_err(go[g0:g0 + n_g], gp.cpu().numpy().astype(wide)) < 1e-6, L
        assert rel_err(co[c0:c0 + n_c], cp.cpu().numpy().astype(wide)) < 1e-6, L


def test_three_launch_eager_timing(gblib, torch_cuda):
    """With stage timing on, a three-launch batch runs eagerly and reports one slice-FFT, one GEMM and one
    conversion launch per direction; the per-bucket form reports its per-bucket launches instead."""
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    lmax = [8, 16, 8, 24]
    b = gblib.Batch(gblib.SO3_REAL, lmax, "tc_bf16x3", "reference", gblib.FLAG_GRAPH)
    g = torch.zeros(b.grid_elems, dtype=torch.float32, device="cuda")
    c = torch.zeros(b.coeff_elems, dtype=torch.float32, device="cuda")
    b.set_timing(True)
    b.forward(g.data_ptr(), c.data_ptr(), s)
    b.inverse(c.data_ptr(), g.data_ptr(), s)
    b.check()
    got = {name: int(n) for name, (ms, n) in b.stage_times(-1).items()}
    assert got == {"fft_slices": 2, "tc_gemm_fwd": 1, "tc_gemm_inv": 1, "coeff_convert": 2}, got
    assert b.graph_kernels(0) == -1
