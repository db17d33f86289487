"""Host-side logic of the drop-in API: containers, index maps, Euler angles,
grid sampling (no GPU)."""
import numpy as np
import pytest

import fftso3_gb300 as fg
from fftso3_gb300.transforms import FFTSO3_complex, FFTS2_real


def test_so3_container_layout_matches_reference_indexing():
    F = fg.FFTSO3_matrix_complex(4)
    assert F.M.size == fg.so3_ncoeff(4) == 5 * (4 * 25 - 1) // 3
    for l in range(5):
        for m in range(-l, l + 1):
            for n in range(-l, l + 1):
                F[l, m, n] = l * 10000 + (m + l) * 100 + (n + l)
    for l in range(5):
        blk = F[l]
        assert blk.shape == (2 * l + 1, 2 * l + 1)
        for m in range(-l, l + 1):
            for n in range(-l, l + 1):
                # F(l,m,n) = M[l](m+l, n+l), column-major packed
                assert blk[m + l, n + l] == F(l, m, n) == l * 10000 + (m + l) * 100 + (n + l)
                assert F.M[fg.so3_index(l, m, n)] == F(l, m, n)
    F[2][0, 0] = 7.0  # writes go through the view
    assert F(2, -2, -2) == 7.0
    with pytest.raises(IndexError):
        F(2, 3, 0)
    with pytest.raises(IndexError):
        F[5]


def test_container_algebra_and_norm():
    rng = np.random.default_rng(0)
    F = fg.FFTSO3_matrix_complex(3)
    G = fg.FFTSO3_matrix_real(3)
    F.setRandom(rng)
    G.setRandom(rng)
    assert np.all(np.abs(F.M.real) <= 1) and np.all(np.abs(G.M) <= 1)
    H = F + G
    assert isinstance(H, fg.FFTSO3_matrix_complex)
    assert np.allclose((H - G).M, F.M)
    assert np.allclose((F * 2.0).M, 2 * F.M)
    assert isinstance(G * 2.0, fg.FFTSO3_matrix_real)
    expect = sum(np.linalg.norm(F[l]) for l in range(4))
    assert abs(F.norm() - expect) < 1e-12
    R = F.real()
    assert isinstance(R, fg.FFTSO3_matrix_real) and np.array_equal(R.M, F.M.real)
    F.setZero()
    assert F.norm() == 0.0
    assert "l=3" in str(G)


def test_s2_container():
    F = fg.FFTS2_matrix_real(3)
    for l in range(4):
        for m in range(-l, l + 1):
            F[l, m] = 100 * l + m
    assert F[2].shape == (5,)
    assert F(3, -3) == 297 and F.M[fg.s2_index(3, -3)] == 297
    with pytest.raises(IndexError):
        F(1, 2)


def test_euler_roundtrip():
    rng = np.random.default_rng(1)
    for _ in range(50):
        a, b, g = rng.uniform(-np.pi, np.pi), rng.uniform(0.01, np.pi - 0.01), rng.uniform(-np.pi, np.pi)
        R = fg.euler323_to_R(a, b, g)
        assert np.allclose(R @ R.T, np.eye(3)) and abs(np.linalg.det(R) - 1) < 1e-12
        a2, b2, g2 = fg.R_to_euler323(R)
        assert np.allclose(fg.euler323_to_R(a2, b2, g2), R, atol=1e-12)
    a, b, g = fg.R_to_euler323(np.eye(3))
    assert b == 0.0 and a == g == 0.0


def test_grid_sampling_orders_axes_like_the_reference():
    t = FFTSO3_complex.__new__(FFTSO3_complex)
    t.__init__(None)
    t.init(3)
    N = 8
    g = t.sample(lambda a, b, c: a + 10 * b + 100 * c)
    assert g.shape == (N, N, N)
    k, j1, j2 = 3, 5, 6
    expect = fg.alpha_j(3, j1) + 10 * fg.beta_k(3, k) + 100 * fg.alpha_j(3, j2)
    assert abs(g[k, j1, j2] - expect) < 1e-12
    # per-point fallback for callbacks that only take scalars
    g2 = t.sample(lambda a, b, c: float(a) + 10 * float(b) + 100 * float(c))
    assert np.allclose(g, g2)
    # one-argument callbacks receive rotation matrices
    g3 = t.sample(lambda R: np.trace(R, axis1=-2, axis2=-1))
    R = fg.euler323_to_R(fg.alpha_j(3, j1), fg.beta_k(3, k), fg.alpha_j(3, j2))
    assert abs(g3[k, j1, j2] - np.trace(R)) < 1e-12
    s = FFTS2_real.__new__(FFTS2_real)
    s.__init__(None)
    s.init(3)
    h = s.sample(lambda th, ph: th + 10 * ph)
    assert h.shape == (N, N) and abs(h[2, 7] - (fg.beta_k(3, 2) + 10 * fg.alpha_j(3, 7))) < 1e-12
