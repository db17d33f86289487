"""The exact inverse (FFTSO3_FLAG_EXACT_INVERSE) of the FP32-data plans (GPU).

SO(3) with l_max <= 255: exact digit sums on the tensor cores, then a
double-float FFT (N = 64..512: the k-contiguous kernels; other N: the generic
line kernels), rounded once to complex64 / float32.  Other plans (S^2, or
FFTSO3_REFINE_FP64=1 at plan creation): the FP64 inverse, rounded once.

Bound, per grid value and component: |g - g_ref| <= 2^-24 |g_ref| + 1e-8 rms(g_ref),
g_ref the oracle's FP64 synthesis of the same (complex64 / float32)
coefficients: the output rounding (at most half an FP32 ulp) plus the digit
truncation of the exact contraction (~1e-9) and the double-float FFT error.
"""
import numpy as np
import pytest

from conftest import s2_coeffs, so3_coeffs
from test_gpu_refine import _with_env

pytestmark = pytest.mark.gpu


def _bound_ok(got, ref):
    rms = np.sqrt(np.mean(np.abs(ref) ** 2))
    parts = [(got.real, ref.real), (got.imag, ref.imag)] if np.iscomplexobj(ref) else [(got, ref)]
    ok = all(bool((np.abs(a - r) <= 2.0 ** -24 * np.abs(r) + 1e-8 * rms).all()) for a, r in parts)
    return ok, float((np.abs(got - ref) / rms).max())


def _exact_inverse(gblib, kind, L, F32, env=None):
    import torch
    b = F32.shape[0]
    flags = gblib.FLAG_EXACT_INVERSE
    p = _with_env(env or {}, lambda: gblib.Plan(kind, L, b, "tc_bf16x3", "stable", flags))
    cplx = kind in (gblib.SO3_COMPLEX, gblib.S2_COMPLEX)
    c = torch.from_numpy(np.ascontiguousarray(F32).ravel()).cuda()
    g = torch.empty(b * p.grid_elems, dtype=torch.complex64 if cplx else torch.float32, device="cuda")
    p.inverse(c.data_ptr(), g.data_ptr(), torch.cuda.current_stream().cuda_stream)
    p.check()
    out = g.cpu().numpy().reshape(b, -1)
    del p
    return out


@pytest.mark.parametrize("kind,L", [("complex", 15), ("complex", 31), ("complex", 47), ("real", 20), ("real", 31),
                                    ("complex", 63)])
def test_exact_inverse_rounds_once(gblib, oracle, kind, L):
    """Batch 9 in chunks of 4 (FFTSO3_REFINE_CHUNK=4): N = 32, 96, 42 run the generic double-float FFT, N = 64
    and 128 the k-contiguous one."""
    cplx = kind == "complex"
    k = gblib.SO3_COMPLEX if cplx else gblib.SO3_REAL
    b = 9
    F = np.stack([so3_coeffs(L, seed=5000 + 13 * L + i, complex_=cplx, decay="pow") for i in range(b)])
    F32 = F.astype(np.complex64 if cplx else np.float32)
    got = _exact_inverse(gblib, k, L, F32, {"FFTSO3_REFINE_CHUNK": "4"})
    for i in range(b):
        Fi = F32[i].astype(np.complex128 if cplx else np.float64)
        ref = oracle.so3_inverse_complex_grid(L, Fi) if cplx else oracle.so3_inverse_real_grid(L, Fi)
        ok, mx = _bound_ok(got[i].astype(ref.dtype), ref.ravel())
        assert ok, (i, mx)


def test_exact_inverse_fp64_fallback(gblib, oracle):
    """FFTSO3_REFINE_FP64=1: the FP64 inverse, rounded once -- the same bound."""
    L, b = 15, 3
    F = np.stack([so3_coeffs(L, seed=5100 + i, decay="pow") for i in range(b)]).astype(np.complex64)
    got = _exact_inverse(gblib, gblib.SO3_COMPLEX, L, F, {"FFTSO3_REFINE_FP64": "1"})
    for i in range(b):
        ref = oracle.so3_inverse_complex_grid(L, F[i].astype(np.complex128)).ravel()
        ok, mx = _bound_ok(got[i].astype(np.complex128), ref)
        assert ok, (i, mx)


@pytest.mark.parametrize("kind", ["complex", "real"])
def test_exact_inverse_s2(gblib, oracle, kind):
    """S^2 plans: the FP64 inverse, rounded once."""
    cplx = kind == "complex"
    L, b = 40, 5
    F = np.stack([s2_coeffs(L, seed=5200 + i, complex_=cplx) for i in range(b)])
    F32 = F.astype(np.complex64 if cplx else np.float32)
    got = _exact_inverse(gblib, gblib.S2_COMPLEX if cplx else gblib.S2_REAL, L, F32)
    for i in range(b):
        Fi = F32[i].astype(np.complex128 if cplx else np.float64)
        ref = (oracle.s2_inverse_complex_grid(L, Fi) if cplx else oracle.s2_inverse_real_grid(L, Fi)).ravel()
        ok, mx = _bound_ok(got[i].astype(ref.dtype), ref)
        assert ok, (i, mx)


@pytest.mark.parametrize("kind,b", [("complex", 5), ("complex", 17), ("real", 17)])
def test_exact_inverse_host_call_equals_device_call(gblib, oracle, kind, b):
    """fftso3_inverse_host on an exact-inverse plan (l_max 31: chunks of 8 functions whose coefficients are copied
    in and whose grids stream out through the two-slot device ring, across chunk boundaries) gives the device
    call's grids bit for bit, into pageable and pinned host memory."""
    import torch
    L = 31
    cplx = kind == "complex"
    k = gblib.SO3_COMPLEX if cplx else gblib.SO3_REAL
    F = np.stack([so3_coeffs(L, seed=5300 + i, complex_=cplx, decay="pow") for i in range(b)])
    F = F.astype(np.complex64 if cplx else np.float32)
    p = gblib.Plan(k, L, b, "tc_bf16x3", "stable", gblib.FLAG_EXACT_INVERSE | gblib.FLAG_REFINE)
    s = torch.cuda.current_stream().cuda_stream
    c = torch.from_numpy(F.ravel()).cuda()
    g = torch.empty(b * p.grid_elems, dtype=torch.complex64 if cplx else torch.float32, device="cuda")
    p.inverse(c.data_ptr(), g.data_ptr(), s)
    p.check()
    want = g.cpu().numpy()
    host = np.ascontiguousarray(F.ravel())
    out = np.empty_like(want)
    p.inverse_host(host.ctypes.data, out.ctypes.data, s)  # pageable
    assert np.array_equal(out, want)
    pin = torch.from_numpy(host).pin_memory()
    pout = torch.empty(want.size, dtype=g.dtype).pin_memory()
    for _ in range(2):  # twice: the ring's slots continue from the previous call
        pout.zero_()
        p.inverse_host(pin.data_ptr(), pout.data_ptr(), s)
        assert np.array_equal(pout.numpy(), want)


def test_exact_inverse_is_more_accurate_than_the_plain_inverse(gblib, oracle):
    """l_max = 63 complex: the plain tensor-core inverse's error is FP32-FFT sized, the exact one's is the output
    rounding."""
    import torch
    L, b = 63, 2
    F = np.stack([so3_coeffs(L, seed=5400 + i, decay="pow") for i in range(b)]).astype(np.complex64)
    plain = gblib.Plan(gblib.SO3_COMPLEX, L, b, "tc_bf16x3", "stable")
    c = torch.from_numpy(F.ravel()).cuda()
    g = torch.empty(b * plain.grid_elems, dtype=torch.complex64, device="cuda")
    plain.inverse(c.data_ptr(), g.data_ptr(), torch.cuda.current_stream().cuda_stream)
    plain.check()
    gp = g.cpu().numpy().reshape(b, -1)
    ge = _exact_inverse(gblib, gblib.SO3_COMPLEX, L, F)
    ref = oracle.so3_inverse_complex_grid(L, F[0].astype(np.complex128)).ravel()
    rms = np.sqrt(np.mean(np.abs(ref) ** 2))
    e_plain = np.abs(gp[0] - ref).max() / rms
    e_exact = np.abs(ge[0] - ref).max() / rms
    assert e_exact <= 2.0 ** -23 * np.abs(ref).max() / rms
    assert e_exact < e_plain
