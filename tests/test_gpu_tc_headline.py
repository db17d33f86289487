"""The headline size, l_max = 255 (512^3 grid): tensor-core split-BF16 path against the
plain FP64 GPU path on the same function, forward, inverse and refined forward (GPU).

Error metric (defined once for the whole suite of precision checks):
  rel_rms = ||a - b||_2 / ||b||_2 over all (l, m, n);
  rel_max = max_l max_mn |a - b| / rms_mn |b|, the per-degree normalisation that
  stays meaningful under the (l+1)^-1.5 spectrum of the inputs.

Bounds asserted here:
  * forward and inverse on the tensor cores, FP32 FFT: rel_rms <= 1e-6 (measured
    about 4.6e-7 forward, 3.4e-7 inverse); the forward's per-degree maximum is
    bounded by 6e-6 (measured about 3.2e-6: the FP32 FFT's rounding, relative to
    the whole grid, seen against the small high-degree coefficients);
  * refined forward (FFTSO3_FLAG_REFINE: F += forward(f - inverse(F)), the inverse
    and the difference in FP64): rel_max <= 1e-6 and rel_rms <= 1e-7.
The FP64 path itself is pinned to the oracle at smaller l_max (test_gpu_so3.py).
"""
import numpy as np
import pytest

from conftest import so3_coeffs

pytestmark = pytest.mark.gpu
L = 255


def per_l_errors(a, b, l_max):
    rms = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    mx = 0.0
    for l in range(l_max + 1):
        o0, o1 = l * (4 * l * l - 1) // 3, (l + 1) * (4 * (l + 1) ** 2 - 1) // 3
        d = np.abs(a[o0:o1] - b[o0:o1]).max()
        r = np.sqrt(np.mean(np.abs(b[o0:o1]) ** 2))
        mx = max(mx, float(d / r))
    return rms, mx


@pytest.fixture(scope="module")
def headline(gblib):
    """FP64 synthesis f of seeded coefficients, the FP64 forward of f, and f as complex64."""
    import torch
    assert torch.cuda.is_available()
    s = torch.cuda.current_stream().cuda_stream
    N = 2 * (L + 1)
    F = so3_coeffs(L, seed=2552, decay="pow")
    p64 = gblib.Plan(gblib.SO3_COMPLEX, L, 1, "fp64", "stable")
    c64 = torch.from_numpy(F).cuda()
    g64 = torch.empty(N ** 3, dtype=torch.complex128, device="cuda")
    o64 = torch.empty_like(c64)
    p64.inverse(c64.data_ptr(), g64.data_ptr(), s)
    p64.forward(g64.data_ptr(), o64.data_ptr(), s)
    p64.check()
    out = {"F": F, "F64": o64.cpu().numpy(), "g32": g64.to(torch.complex64), "g64_host": g64.cpu().numpy()}
    del p64, c64, g64, o64
    torch.cuda.empty_cache()
    return out


def _tc_forward(gblib, grid32, flags):
    import torch
    s = torch.cuda.current_stream().cuda_stream
    p = gblib.Plan(gblib.SO3_COMPLEX, L, 1, "tc_bf16x3", "stable", flags)
    C = p.coeff_elems
    c = torch.empty(C, dtype=torch.complex64, device="cuda")
    p.forward(grid32.data_ptr(), c.data_ptr(), s)
    p.check()
    out = c.cpu().numpy().astype(np.complex128)
    del p
    torch.cuda.empty_cache()
    return out


def test_tc_forward_vs_fp64_lmax255(gblib, headline):
    rms, mx = per_l_errors(_tc_forward(gblib, headline["g32"], 0), headline["F64"], L)
    assert rms <= 1e-6, rms
    assert mx <= 6e-6, mx


def test_tc_inverse_vs_fp64_lmax255(gblib, headline):
    import torch
    s = torch.cuda.current_stream().cuda_stream
    p = gblib.Plan(gblib.SO3_COMPLEX, L, 1, "tc_bf16x3", "stable")
    c = torch.from_numpy(headline["F"].astype(np.complex64)).cuda()
    g = torch.empty(p.grid_elems, dtype=torch.complex64, device="cuda")
    p.inverse(c.data_ptr(), g.data_ptr(), s)
    p.check()
    ref = headline["g64_host"]
    got = g.cpu().numpy().astype(np.complex128)
    rms = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    assert rms <= 1e-6, rms


def test_tc_refined_forward_vs_fp64_lmax255(gblib, headline):
    rms, mx = per_l_errors(_tc_forward(gblib, headline["g32"], gblib.FLAG_REFINE), headline["F64"], L)
    assert mx <= 1e-6, mx
    assert rms <= 1e-7, rms
