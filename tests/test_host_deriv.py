"""Real harmonics and the derivative operators of the reference (host math, no GPU).

Pinned against the oracle's restatement of real_harmonics / wigner_d by central
differences: d/dt U(R exp(t e_i)) = U(R) u_i and d/dt D(R exp(t e_i)) = D(R) u_i
(fdcl_FFTSO3.cpp:417-453, :1577-1645; the reference checks them the same way at
R = I, :455-492, :1648-1681)."""
import numpy as np
import pytest

import fftso3_gb300 as fg
from fftso3_gb300.transforms import real_from_wigner_D

L = 6


def _U_oracle(oracle, R):
    a, b, g = fg.R_to_euler323(R)
    return fg.FFTSO3_matrix_real(L, data=oracle.so3_real_harmonics(L, a, b, g))


def _D_oracle(oracle, R):
    a, b, g = fg.R_to_euler323(R)
    d = fg.FFTSO3_matrix_real(L, data=oracle.wigner_d(b, L))
    D = fg.FFTSO3_matrix_complex(L)
    for l in range(L + 1):
        m = np.arange(-l, l + 1)
        D[l] = d[l] * np.exp(-1j * m * a)[:, None] * np.exp(-1j * m * g)[None, :]
    return D


def test_real_harmonics_from_wigner_D(oracle):
    R = fg.euler323_to_R(0.4, 1.1, -0.7)
    U = real_from_wigner_D(_D_oracle(oracle, R))
    Uo = _U_oracle(oracle, R)
    for l in range(L + 1):
        assert np.allclose(U[l], Uo[l], atol=1e-12)


# generic rotations: at beta = 0 the 3-2-3 angles of R exp(t e_3) lose the sign of t
@pytest.mark.parametrize("R", [fg.euler323_to_R(0.3, 0.9, 2.1), fg.euler323_to_R(-2.0, 2.5, 0.4)])
def test_deriv_real_harmonics(oracle, R):
    u = fg.FFTSO3_real(L).deriv_real_harmonics()
    U = _U_oracle(oracle, R)
    h = 1e-5
    for i in range(1, 4):
        e = np.zeros(3)
        e[i - 1] = h
        Up, Um = _U_oracle(oracle, R @ fg.expm_SO3(e)), _U_oracle(oracle, R @ fg.expm_SO3(-e))
        for l in range(1, L + 1):
            num = (Up[l] - Um[l]) / (2 * h)
            ana = U[l] @ u[i][l]
            assert np.linalg.norm(num - ana) <= 1e-7 * max(1.0, np.linalg.norm(ana)), (i, l)


@pytest.mark.parametrize("R", [fg.euler323_to_R(-1.0, 0.6, 0.2), fg.euler323_to_R(1.3, 1.9, -2.2)])
def test_deriv_wigner_D(oracle, R):
    u = fg.FFTSO3_complex(L).deriv_wigner_D()
    D = _D_oracle(oracle, R)
    h = 1e-5
    for i in range(1, 4):
        e = np.zeros(3)
        e[i - 1] = h
        Dp, Dm = _D_oracle(oracle, R @ fg.expm_SO3(e)), _D_oracle(oracle, R @ fg.expm_SO3(-e))
        for l in range(1, L + 1):
            num = (Dp[l] - Dm[l]) / (2 * h)
            ana = D[l] @ u[i][l]
            assert np.linalg.norm(num - ana) <= 1e-7 * max(1.0, np.linalg.norm(ana)), (i, l)
