"""Clebsch-Gordan coefficients (host math, no GPU): orthogonality, the product
rules of Wigner-D and real harmonics built from the oracle's Wigner-d / real
harmonics (the reference's check_Clebsch_Gordon, fdcl_FFTSO3.cpp:1683+, tests
the real rule at (l1, l2) = (3, 5)), and known closed-form values."""
import numpy as np
import pytest

import fftso3_gb300 as fg
from fftso3_gb300.clebsch_gordan import Clebsch_Gordon_complex, Clebsch_Gordon_real


def _D(oracle, L, a, b, g):
    d = fg.FFTSO3_matrix_real(L, data=oracle.wigner_d(b, L))
    out = []
    for l in range(L + 1):
        m = np.arange(-l, l + 1)
        out.append(d[l] * np.exp(-1j * m * a)[:, None] * np.exp(-1j * m * g)[None, :])
    return out


def _block(mats, lo, hi):
    n = sum(mats[l].shape[0] for l in range(lo, hi + 1))
    B = np.zeros((n, n), complex)
    i = 0
    for l in range(lo, hi + 1):
        w = mats[l].shape[0]
        B[i:i + w, i:i + w] = mats[l]
        i += w
    return B


@pytest.mark.parametrize("l1,l2", [(0, 0), (1, 1), (2, 1), (3, 5), (6, 4)])
def test_complex_product_rule(oracle, l1, l2):
    cg = Clebsch_Gordon_complex()
    cg.compute_host(l1, l2)
    n = cg.C.shape[0]
    assert np.allclose(cg.C.T @ cg.C, np.eye(n), atol=1e-12)
    D = _D(oracle, l1 + l2, 0.7, 1.3, -0.4)
    lhs = np.kron(D[l1], D[l2])
    rhs = cg.C @ _block(D, abs(l1 - l2), l1 + l2) @ cg.C.T
    assert np.allclose(lhs, rhs, atol=1e-11)


@pytest.mark.parametrize("l1,l2", [(3, 5), (2, 2)])
def test_real_product_rule(oracle, l1, l2):
    cg = Clebsch_Gordon_real()
    cg.compute_host(l1, l2)
    L = l1 + l2
    a, b, g = 2.1, 0.8, 1.7
    U = fg.FFTSO3_matrix_real(L, data=oracle.so3_real_harmonics(L, a, b, g))
    Ul = [U[l] for l in range(L + 1)]
    lhs = np.kron(Ul[l1], Ul[l2])
    rhs = cg.c @ _block(Ul, abs(l1 - l2), L) @ cg.c.conj().T
    assert np.allclose(lhs, rhs, atol=1e-11)


def test_known_values():
    cg = Clebsch_Gordon_complex(1, 1)
    cg.compute_host(1, 1)
    s2 = 1 / np.sqrt(2)
    assert np.isclose(cg(2, 2, 1, 1, 1, 1), 1.0)
    assert np.isclose(cg(2, 1, 1, 1, 1, 0), s2) and np.isclose(cg(2, 1, 1, 0, 1, 1), s2)
    assert np.isclose(cg(0, 0, 1, 1, 1, -1), 1 / np.sqrt(3))
    assert np.isclose(abs(cg(1, 0, 1, 1, 1, -1)), s2)
    with pytest.raises(ValueError):
        cg(3, 0, 1, 0, 1, 0)
