"""The residual refinement (FFTSO3_FLAG_REFINE) of the tensor-core SO(3) forward (GPU).

F += forward(f - inverse(F)): for SO(3) with l_max <= 255 the inverse runs on the
tensor cores with exact digit sums (BF16 digit planes, FP32 TMEM accumulators that
never round).  For N = 64..512 (l_max 31, 63, 127, 255) the step is spectral: the
samples' FFT in double-float, F0 from its FP32 part, and the residual
FFT(f) - N^2 H(F0) in the pencil domain; otherwise a double-float FFT of the
synthesis and the residual against the FP32 samples on the grid.
FFTSO3_REFINE_FP64=1 at plan creation selects the FP64 inverse (grid form).  Either
way the refined coefficients are the FP64 forward of the FP32 samples up to the
complex64 rounding of the output.

Error metric: rel_rms = ||a - b|| / ||b||; rel_max = max_l max_mn |a - b| / rms_mn |b|.
Bounds: rel_rms <= 1e-7 and rel_max <= 1e-6 against the oracle's forward of the same
FP32 samples (measured ~3e-8 / ~2e-7 at l_max = 255).
"""
import os

import numpy as np
import pytest

from conftest import so3_coeffs

pytestmark = pytest.mark.gpu


def per_l_errors(a, b, l_max):
    rms = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    mx = 0.0
    for l in range(l_max + 1):
        o0, o1 = l * (4 * l * l - 1) // 3, (l + 1) * (4 * (l + 1) ** 2 - 1) // 3
        d = np.abs(a[o0:o1] - b[o0:o1]).max()
        r = np.sqrt(np.mean(np.abs(b[o0:o1]) ** 2))
        mx = max(mx, float(d / r))
    return rms, mx


def _with_env(env, make):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return make()
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def _refined(gblib, kind, L, grids32, fp64_inverse=False, chunk=None):
    import torch
    s = torch.cuda.current_stream().cuda_stream
    b = grids32.shape[0]
    env = {}
    if fp64_inverse:
        env["FFTSO3_REFINE_FP64"] = "1"
    if chunk:
        env["FFTSO3_REFINE_CHUNK"] = str(chunk)
    p = _with_env(env, lambda: gblib.Plan(kind, L, b, "tc_bf16x3", "stable", gblib.FLAG_REFINE))
    cplx = kind == gblib.SO3_COMPLEX
    g = torch.from_numpy(np.ascontiguousarray(grids32).ravel()).cuda()
    c = torch.empty(b * p.coeff_elems, dtype=torch.complex64 if cplx else torch.float32, device="cuda")
    p.forward(g.data_ptr(), c.data_ptr(), s)
    p.check()
    out = c.cpu().numpy().astype(np.complex128 if cplx else np.float64).reshape(b, -1)
    del p
    return out


@pytest.mark.parametrize("kind,L", [("complex", 15), ("complex", 31), ("real", 31), ("complex", 47), ("real", 20)])
def test_refined_forward_matches_oracle(gblib, oracle, kind, L):
    """Batch 9 in refinement chunks of 4 (4 + 4 + 1 functions, FFTSO3_REFINE_CHUNK=4)."""
    cplx = kind == "complex"
    k = gblib.SO3_COMPLEX if cplx else gblib.SO3_REAL
    N = 2 * (L + 1)
    b = 9
    grids, refs = [], []
    for i in range(b):
        F = so3_coeffs(L, seed=4000 + 17 * L + i, complex_=cplx, decay="pow")
        if cplx:
            g = oracle.so3_inverse_complex_grid(L, F).astype(np.complex64)
            ref = oracle.so3_forward_complex(L, g.astype(np.complex128))
        else:
            g = oracle.so3_inverse_real_grid(L, F).astype(np.float32)
            ref = oracle.so3_forward_real(L, g.astype(np.float64))
        grids.append(g.reshape(N, N, N))
        refs.append(ref)
    out = _refined(gblib, k, L, np.stack(grids), chunk=4)
    for i in range(b):
        rms, mx = per_l_errors(out[i], refs[i], L)
        assert rms <= 1e-7 and mx <= 1e-6, (i, rms, mx)


def test_exact_and_fp64_refinement_agree(gblib, oracle):
    """The tensor-core exact inverse and the FP64 inverse give the same refined coefficients (to the complex64
    rounding of the output and the ~1e-9 of the exact inverse)."""
    L = 31
    N = 2 * (L + 1)
    grids = []
    for i in range(3):
        F = so3_coeffs(L, seed=4500 + i, decay="pow")
        grids.append(oracle.so3_inverse_complex_grid(L, F).astype(np.complex64).reshape(N, N, N))
    grids = np.stack(grids)
    a = _refined(gblib, gblib.SO3_COMPLEX, L, grids)
    b = _refined(gblib, gblib.SO3_COMPLEX, L, grids, fp64_inverse=True)
    for i in range(3):
        rms, mx = per_l_errors(a[i], b[i], L)
        assert rms <= 1e-7 and mx <= 1e-6, (i, rms, mx)


@pytest.mark.parametrize("L,b", [(15, 3), (31, 9)])
@pytest.mark.parametrize("kind", ["complex", "real"])
def test_refined_host_call_equals_device_call(gblib, oracle, kind, L, b):
    """fftso3_forward_host on a refined plan (samples staged once into the residual buffer, which the residual --
    grid form, l_max 15 -- or the FFT remainders -- spectral form, l_max 31, the samples copied in pieces of 4
    functions under the FFT of the previous piece -- then overwrite chunk by chunk) gives the same coefficients,
    bit for bit, as fftso3_forward on device buffers; pageable and pinned host samples, and the host samples are
    left unchanged."""
    import torch
    cplx = kind == "complex"
    k = gblib.SO3_COMPLEX if cplx else gblib.SO3_REAL
    N = 2 * (L + 1)
    gs = []
    for i in range(b):
        F = so3_coeffs(L, seed=4700 + i, complex_=cplx, decay="pow")
        g = oracle.so3_inverse_complex_grid(L, F) if cplx else oracle.so3_inverse_real_grid(L, F)
        gs.append(g.astype(np.complex64 if cplx else np.float32).ravel())
    host = np.ascontiguousarray(np.concatenate(gs))
    keep = host.copy()
    p = gblib.Plan(k, L, b, "tc_bf16x3", "stable", gblib.FLAG_REFINE)
    s = torch.cuda.current_stream().cuda_stream
    dt = torch.complex64 if cplx else torch.float32
    dev = torch.from_numpy(host).cuda()
    cd = torch.empty(b * p.coeff_elems, dtype=dt, device="cuda")
    p.forward(dev.data_ptr(), cd.data_ptr(), s)
    p.check()
    want = cd.cpu().numpy()
    out = np.empty_like(want)
    p.forward_host(host.ctypes.data, out.ctypes.data, s)  # pageable
    assert np.array_equal(out, want)
    assert np.array_equal(host, keep)
    pin = torch.from_numpy(host).pin_memory()
    pout = torch.empty(want.size, dtype=dt).pin_memory()
    p.forward_host(pin.data_ptr(), pout.data_ptr(), s)  # pinned
    assert np.array_equal(pout.numpy(), want)
    assert N ** 3 * b == host.size
