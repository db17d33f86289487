"""The Python walkthrough of the integration notes, run as written (GPU).

Checks that the calls a reference user is shown work and agree with each other: README example0
through FFTSO3_real, a callback forward at l_max = 127 with the stable recursion, grid synthesis,
and single-point and batched point evaluation (equal to each other and, at grid nodes, to the grid).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_python_walkthrough():
    import fftso3_gb300 as fftso3

    R = fftso3.FFTSO3_real(2)
    F = R.forward_transform(lambda Rm: np.trace(Rm, axis1=-2, axis2=-1))
    assert np.abs(F[1] - np.eye(3) / 3).max() < 1e-15
    assert abs(R.inverse_transform(F, np.eye(3)) - 3.0) < 1e-13

    L = 127
    C = fftso3.FFTSO3_complex(L, recursion="stable")
    G = C.forward_transform(lambda a, b, g: np.cos(a) * np.sin(b))
    grid = C.inverse_grid(G)
    # cos(alpha) sin(beta) is band-limited at l = 1: the synthesis returns it on the grid
    k, j1, j2 = 37, 5, 200
    a, b = fftso3.alpha_j(L, j1), fftso3.beta_k(L, k)
    assert abs(grid[k, j1, j2] - np.cos(a) * np.sin(b)) < 1e-12
    val = C.inverse_transform(G, 0.1, 0.2, 0.3)
    assert abs(val - np.cos(0.1) * np.sin(0.2)) < 1e-12
    abg = np.array([[0.1, 0.2, 0.3], [a, b, fftso3.alpha_j(L, j2)], [-2.0, 3.0, 1.0]])
    vals = C.inverse_points(G, abg)
    assert abs(vals[0] - val) < 1e-13
    assert abs(vals[1] - grid[k, j1, j2]) < 1e-12
    assert abs(vals[2] - np.cos(-2.0) * np.sin(3.0)) < 1e-12
