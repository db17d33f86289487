"""SO(3) parity of the CUDA library against the oracle (GPU).

Tolerances: the FP64 path must match the reference's algorithm within 1e-12
relative (||a - b||_2 / ||b||_2 over all coefficients or grid values); the
faithful Wigner-d table must match it bit for bit.
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


def gpu_wigner_d(gblib, beta, L, recursion):
    d = np.zeros((L + 1) * (4 * (L + 1) ** 2 - 1) // 3)
    gblib.check(gblib.lib().fftso3_wigner_d(float(beta), L, recursion, d.ctypes.data_as(gblib._dp)))
    return d


@pytest.mark.parametrize("L", [1, 3, 16, 127])
def test_wigner_d_faithful_is_bitwise(gblib, oracle, L):
    N = 2 * (L + 1)
    betas = [oracle.beta_k(L, k) for k in (0, 1, N // 2, N - 2, N - 1)] + [0.3, 2.0, -1.1]
    for beta in betas:
        assert np.array_equal(gpu_wigner_d(gblib, beta, L, gblib.RECURSION_REFERENCE), oracle.wigner_d(beta, L))


@pytest.mark.parametrize("L", [16, 127, 255])
def test_wigner_d_stable_is_orthogonal(gblib, oracle, L):
    N = 2 * (L + 1)
    for k in (0, N // 3, N - 1):
        beta = oracle.beta_k(L, k)
        d = gpu_wigner_d(gblib, beta, L, gblib.RECURSION_STABLE)
        for l in sorted({1, L // 2, L - 1, L}):
            o = l * (4 * l * l - 1) // 3
            M = d[o:o + (2 * l + 1) ** 2].reshape(2 * l + 1, 2 * l + 1, order="F")
            assert np.abs(M.T @ M - np.eye(2 * l + 1)).max() < 1e-11, (k, l)
        if L <= 64:  # no underflow in the reference there: both agree
            assert np.abs(d - oracle.wigner_d(beta, L)).max() < 1e-12


def _plan(gblib, kind, L, batch=1, recursion="reference", precision="fp64"):
    return gblib.Plan(kind, L, batch, precision, recursion)


def _fwd(torch, plan, grid_np, complex_=True):
    g = torch.from_numpy(np.ascontiguousarray(grid_np)).cuda()
    out = torch.empty(plan.batch * plan.coeff_elems, dtype=torch.complex128 if complex_ else torch.float64,
                      device="cuda")
    plan.forward(g.data_ptr(), out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _inv(torch, plan, F_np, complex_=True):
    c = torch.from_numpy(np.ascontiguousarray(F_np)).cuda()
    out = torch.empty(plan.batch * plan.grid_elems, dtype=torch.complex128 if complex_ else torch.float64,
                      device="cuda")
    plan.inverse(c.data_ptr(), out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("L", [0, 1, 2, 5, 16])
def test_so3_complex_matches_oracle_small(gblib, oracle, torch_cuda, L):
    N = 2 * (L + 1)
    F = so3_coeffs(L, seed=L)
    g_ref = oracle.so3_inverse_complex_grid(L, F)
    p = _plan(gblib, gblib.SO3_COMPLEX, L)
    g = _inv(torch_cuda, p, F).reshape(N, N, N)
    assert rel_err(g, g_ref) < TOL
    G_ref = oracle.so3_forward_complex(L, g_ref)
    G = _fwd(torch_cuda, p, g_ref)
    assert rel_err(G, G_ref) < TOL
    assert rel_err(G, F) < 1e-12


@pytest.mark.parametrize("L", [0, 1, 5, 16])
def test_so3_real_matches_oracle_small(gblib, oracle, torch_cuda, L):
    N = 2 * (L + 1)
    F = so3_coeffs(L, seed=100 + L, complex_=False)
    g_ref = oracle.so3_inverse_real_grid(L, F)
    p = _plan(gblib, gblib.SO3_REAL, L)
    g = _inv(torch_cuda, p, F, complex_=False).reshape(N, N, N)
    assert rel_err(g, g_ref) < TOL
    G_ref = oracle.so3_forward_real(L, g_ref)
    G = _fwd(torch_cuda, p, g_ref, complex_=False)
    assert rel_err(G, G_ref) < TOL
    assert rel_err(G, F) < 1e-12


def test_so3_complex_l127_matches_reference_path(gblib, oracle, torch_cuda):
    """Plain FP64 GPU path at l_max = 127 (256^3 grid) vs the reference's
    algorithm, both with the reference's Wigner-d recursion."""
    L, N = 127, 256
    F = so3_coeffs(L, seed=1)
    g_ref = oracle.so3_inverse_complex_grid(L, F)
    p = _plan(gblib, gblib.SO3_COMPLEX, L)
    g = _inv(torch_cuda, p, F).reshape(N, N, N)
    assert rel_err(g, g_ref) < TOL
    G_ref = oracle.so3_forward_complex(L, g_ref)
    G = _fwd(torch_cuda, p, g_ref)
    assert rel_err(G, G_ref) < TOL


def test_so3_real_l127_matches_reference_path(gblib, oracle, torch_cuda):
    L, N = 127, 256
    F = so3_coeffs(L, seed=2, complex_=False)
    g_ref = oracle.so3_inverse_real_grid(L, F)
    p = _plan(gblib, gblib.SO3_REAL, L)
    g = _inv(torch_cuda, p, F, complex_=False).reshape(N, N, N)
    assert rel_err(g, g_ref) < TOL
    G_ref = oracle.so3_forward_real(L, g_ref)
    G = _fwd(torch_cuda, p, g_ref, complex_=False)
    assert rel_err(G, G_ref) < TOL


@pytest.mark.parametrize("L", [96, 127, 255])
def test_so3_stable_roundtrip(gblib, torch_cuda, L):
    """Size-independent property at full sizes: inverse then forward returns F
    (band-limited), with the stable recursion (the reference's own recursion
    cannot round-trip above l_max ~ 90 because of the seed underflow)."""
    torch = torch_cuda
    F = so3_coeffs(L, seed=3, decay="pow")
    p = _plan(gblib, gblib.SO3_COMPLEX, L, recursion="stable")
    c = torch.from_numpy(F).cuda()
    g = torch.empty(p.grid_elems, dtype=torch.complex128, device="cuda")
    out = torch.empty_like(c)
    s = torch.cuda.current_stream().cuda_stream
    p.inverse(c.data_ptr(), g.data_ptr(), s)
    p.forward(g.data_ptr(), out.data_ptr(), s)
    torch.cuda.synchronize()
    assert rel_err(out.cpu().numpy(), F) < 1e-11
    del g


def test_reference_recursion_cannot_roundtrip_l127(gblib, torch_cuda):
    """The faithful mode reproduces the reference's loss of accuracy at l_max = 127."""
    torch = torch_cuda
    L = 127
    F = so3_coeffs(L, seed=4)
    p = _plan(gblib, gblib.SO3_COMPLEX, L)
    c = torch.from_numpy(F).cuda()
    g = torch.empty(p.grid_elems, dtype=torch.complex128, device="cuda")
    out = torch.empty_like(c)
    s = torch.cuda.current_stream().cuda_stream
    p.inverse(c.data_ptr(), g.data_ptr(), s)
    p.forward(g.data_ptr(), out.data_ptr(), s)
    torch.cuda.synchronize()
    assert rel_err(out.cpu().numpy(), F) > 1e-6


def test_so3_batch_equals_single(gblib, oracle, torch_cuda):
    L, N, b = 7, 16, 3
    Fs = np.stack([so3_coeffs(L, seed=20 + i) for i in range(b)])
    pb = _plan(gblib, gblib.SO3_COMPLEX, L, batch=b)
    gb = _inv(torch_cuda, pb, Fs.ravel()).reshape(b, N, N, N)
    Gb = _fwd(torch_cuda, pb, gb).reshape(b, -1)
    for i in range(b):
        assert rel_err(gb[i], oracle.so3_inverse_complex_grid(L, Fs[i])) < TOL
        assert rel_err(Gb[i], Fs[i]) < 1e-12


@pytest.mark.parametrize("kind", ["complex", "real"])
def test_point_evaluation_matches_reference(gblib, oracle, kind):
    import fftso3_gb300 as fg
    L = 12
    rng = np.random.default_rng(9)
    if kind == "complex":
        T = fg.FFTSO3_complex(L)
        F = fg.FFTSO3_matrix_complex(L, data=so3_coeffs(L, 11))
        ref = oracle.so3_inverse_complex_point
    else:
        T = fg.FFTSO3_real(L)
        F = fg.FFTSO3_matrix_real(L, data=so3_coeffs(L, 12, complex_=False))
        ref = oracle.so3_inverse_real_point
    pts = np.column_stack([rng.uniform(-np.pi, np.pi, 20), rng.uniform(0.05, np.pi - 0.05, 20),
                           rng.uniform(-np.pi, np.pi, 20)])
    got = T.inverse_points(F, pts) if kind == "complex" else np.array([T.inverse_transform(F, *p) for p in pts])
    want = np.array([ref(L, F.M, *p) for p in pts])
    assert rel_err(got, want) < 1e-12


@pytest.mark.parametrize("recursion", ["reference", "stable"])
def test_point_evaluation_partial_warp_many_parts(gblib, oracle, recursion):
    """Point evaluation with a partial last warp of points and the degrees split into many parts
    (45 points at l_max = 37: two batches of 32 points, 32 degree parts), points near both poles,
    and a one-point call; both recursions against the oracle (no underflow at this l_max, so the
    stable recursion agrees with the reference's to rounding)."""
    import fftso3_gb300 as fg
    L = 37
    rng = np.random.default_rng(21)
    T = fg.FFTSO3_complex(L, recursion=recursion)
    F = fg.FFTSO3_matrix_complex(L, data=so3_coeffs(L, 13))
    pts = np.column_stack([rng.uniform(-np.pi, np.pi, 45), rng.uniform(0.0, np.pi, 45),
                           rng.uniform(-np.pi, np.pi, 45)])
    pts[0, 1], pts[1, 1] = 1e-3, np.pi - 1e-3
    got = T.inverse_points(F, pts)
    want = np.array([oracle.so3_inverse_complex_point(L, F.M, *p) for p in pts])
    assert rel_err(got, want) < TOL
    one = T.inverse_points(F, pts[5:6])
    assert abs(one[0] - want[5]) < TOL * abs(want[5])
    more = T.inverse_points(F, np.concatenate([pts, pts[::-1]]))  # a larger call reuses the plan's scratch
    assert rel_err(more, np.concatenate([want, want[::-1]])) < TOL


@pytest.mark.parametrize("L", [0, 1, 2])
def test_point_evaluation_smallest_degrees(gblib, oracle, L):
    """Point evaluation at l_max = 0, 1, 2 (the special seeds of m0 = 0, 1 and an empty or one-row
    recursion table), SO(3) and S^2, against the oracle."""
    import fftso3_gb300 as fg
    rng = np.random.default_rng(40 + L)
    pts = np.column_stack([rng.uniform(-np.pi, np.pi, 7), rng.uniform(0.0, np.pi, 7), rng.uniform(-np.pi, np.pi, 7)])
    F = fg.FFTSO3_matrix_complex(L, data=so3_coeffs(L, 50 + L))
    got = fg.FFTSO3_complex(L).inverse_points(F, pts)
    want = np.array([oracle.so3_inverse_complex_point(L, F.M, *p) for p in pts])
    assert rel_err(got, want) < TOL
    C2 = (L + 1) ** 2
    G = fg.FFTS2_matrix_complex(L, data=rng.standard_normal(C2) + 1j * rng.standard_normal(C2))
    got = fg.FFTS2_complex(L).inverse_points(G, pts[:, 1:])
    want = np.array([oracle.s2_inverse_complex_point(L, G.M, *p) for p in pts[:, 1:]])
    assert rel_err(got, want) < TOL


def test_python_api_example0(gblib):
    """README example0 through the drop-in API on the GPU: tr R -> F^1 = I/3, f(I) = 3."""
    import fftso3_gb300 as fg
    R = fg.FFTSO3_real(2)
    F = R.forward_transform(lambda Rm: np.trace(Rm, axis1=-2, axis2=-1))
    assert np.abs(F[1] - np.eye(3) / 3).max() < 1e-15
    assert abs(F[0][0, 0]) < 1e-15 and np.abs(F[2]).max() < 1e-15
    assert abs(R.inverse_transform(F, np.eye(3)) - 3.0) < 1e-13
    C = fg.FFTSO3_complex(5)
    assert C.check_transform(np.random.default_rng(0)) < 1e-10
    assert fg.FFTSO3_real(5).check_transform(np.random.default_rng(1)) < 1e-10


def test_host_entry_points_equal_device_entry_points(gblib, torch_cuda):
    L = 9
    F = so3_coeffs(L, seed=5)
    p = _plan(gblib, gblib.SO3_COMPLEX, L)
    g_dev = _inv(torch_cuda, p, F)
    g_host = np.empty_like(g_dev)
    Fc = np.ascontiguousarray(F)
    p.inverse_host(Fc.ctypes.data, g_host.ctypes.data)
    assert np.array_equal(g_dev, g_host)
    G_host = np.empty_like(Fc)
    p.forward_host(g_host.ctypes.data, G_host.ctypes.data)
    assert np.array_equal(G_host, _fwd(torch_cuda, p, g_host))


def test_bad_calls_raise(gblib):
    p = _plan(gblib, gblib.SO3_COMPLEX, 4)
    with pytest.raises(gblib.FFTSO3Error):
        p.forward(0, 0)
    pts = np.zeros(3)
    with pytest.raises(gblib.FFTSO3Error):
        p.inverse_points(1, 5, pts.ctypes.data_as(gblib._dp), 1, pts.ctypes.data)


def test_check_clebsch_gordon_and_derivatives(gblib):
    """The reference's check members on the GPU-computed real harmonics / Wigner D."""
    import fftso3_gb300 as fg
    assert fg.FFTSO3_real(8).check_Clebsch_Gordon(rng=1) < 1e-10
    assert fg.FFTSO3_real(6).check_deriv_real_harmonics() < 1e-9
    assert fg.FFTSO3_complex(6).check_deriv_wigner_D() < 1e-9
