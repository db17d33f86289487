"""S^2 -> SO(3) correlation (spherical shape matching) and grid arg-max (GPU).

J(R) = sum_l G[l]^T U^l(R) F[l] on the Euler grid (the cost of the reference's
example/example3_SSM.hpp) against the oracle's real harmonics at sampled grid
rotations (FP64: 1e-12 relative); the arg-max recovers a rotation placed on the grid.
"""
import numpy as np
import pytest

from conftest import rel_err, s2_coeffs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _J_oracle(oracle, L, F, G, a, b, g):
    U = oracle.so3_real_harmonics(L, a, b, g)
    J = 0.0
    for l in range(L + 1):
        W = 2 * l + 1
        Ul = U[oracle.so3_index(l, -l, -l):oracle.so3_index(l, -l, -l) + W * W].reshape(W, W, order="F")
        J += G[l * l:l * l + W] @ Ul @ F[l * l:l * l + W]
    return J


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("tc_bf16x3", 1e-6), ("fp32", 1e-6)])
def test_correlation_grid_matches_oracle(gblib, oracle, torch_cuda, precision, tol):
    torch = torch_cuda
    L = 8
    N = 2 * (L + 1)
    F = s2_coeffs(L, seed=1800, complex_=False)
    G = s2_coeffs(L, seed=1801, complex_=False)
    p = gblib.Plan(gblib.SO3_REAL, L, 1, precision, "reference")
    dt = torch.float64 if precision == "fp64" else torch.float32
    f = torch.from_numpy(F).cuda().to(dt)
    g = torch.from_numpy(G).cuda().to(dt)
    grid = torch.empty(N ** 3, dtype=dt, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    p.correlate_s2(f.data_ptr(), g.data_ptr(), grid.data_ptr(), s)
    p.check()
    J = grid.cpu().numpy().astype(np.float64).reshape(N, N, N)
    rng = np.random.default_rng(5)
    pts = rng.integers(0, N, size=(24, 3))
    ref = np.array([_J_oracle(oracle, L, F, G, oracle.alpha_j(L, j1), oracle.beta_k(L, k), oracle.alpha_j(L, j2))
                    for k, j1, j2 in pts])
    got = np.array([J[k, j1, j2] for k, j1, j2 in pts])
    assert rel_err(got, ref) < tol


def test_shape_matching_recovers_grid_rotation(gblib, oracle, torch_cuda):
    """G[l] = U^l(R_true) F[l] (the rotated shape of the reference example); the correlation's
    arg-max is R_true when R_true lies on the grid."""
    import fftso3_gb300 as fg
    L = 10
    N = 2 * (L + 1)
    F = s2_coeffs(L, seed=1900, complex_=False)
    k, j1, j2 = 7, 3, 15
    a, b, g = oracle.alpha_j(L, j1), oracle.beta_k(L, k), oracle.alpha_j(L, j2)
    U = oracle.so3_real_harmonics(L, a, b, g)
    G = np.zeros_like(F)
    for l in range(L + 1):
        W = 2 * l + 1
        Ul = U[oracle.so3_index(l, -l, -l):oracle.so3_index(l, -l, -l) + W * W].reshape(W, W, order="F")
        G[l * l:l * l + W] = Ul @ F[l * l:l * l + W]
    Fm = fg.FFTS2_matrix_real(L)
    Gm = fg.FFTS2_matrix_real(L)
    Fm.M[:] = F
    Gm.M[:] = G
    J, abg, R = fg.correlate_s2(Fm, Gm)
    assert np.unravel_index(np.argmax(J), J.shape) == (k, j1, j2)
    assert np.allclose(abg, (a, b, g))
    assert np.allclose(R, fg.euler323_to_R(a, b, g))


def test_correlation_gradient_grid(gblib, oracle, torch_cuda):
    """dJ_i on the grid (correlate_s2(gradient=True)) against central differences of the
    oracle's J at R exp(+-h e_i), at sampled grid rotations."""
    import fftso3_gb300 as fg
    L = 6
    N = 2 * (L + 1)
    F = s2_coeffs(L, seed=2000, complex_=False)
    G = s2_coeffs(L, seed=2001, complex_=False)
    Fm, Gm = fg.FFTS2_matrix_real(L), fg.FFTS2_matrix_real(L)
    Fm.M[:] = F
    Gm.M[:] = G
    J, _, _, dJ = fg.correlate_s2(Fm, Gm, gradient=True)
    h = 1e-5
    rng = np.random.default_rng(9)
    for k, j1, j2 in rng.integers(0, N, size=(6, 3)):
        R = fg.euler323_to_R(oracle.alpha_j(L, j1), oracle.beta_k(L, k), oracle.alpha_j(L, j2))
        for i in range(3):
            e = np.zeros(3)
            e[i] = h
            Jp = _J_oracle(oracle, L, F, G, *fg.R_to_euler323(R @ fg.expm_SO3(e)))
            Jm = _J_oracle(oracle, L, F, G, *fg.R_to_euler323(R @ fg.expm_SO3(-e)))
            num = (Jp - Jm) / (2 * h)
            assert abs(dJ[i, k, j1, j2] - num) <= 1e-6 * max(1.0, abs(num)), (i, k, j1, j2)
