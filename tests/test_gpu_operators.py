"""Clebsch-Gordan tables and directional derivatives on the GPU (fftso3_clebsch_gordan,
fftso3_derivative) against the host restatements and the reference's check identities.

Tolerances: Clebsch-Gordan entries (|C| <= 1) within 1e-12 of the numpy recursion for pairs up
to (9, 7); the reference's single downward recursion (reproduced on both sides) loses accuracy for
larger degrees -- orthogonality 6.7e-8 at (20, 15), 0.3 at (30, 30) -- so at (20, 15) the two agree
only to 1e-6, the recursion's own error; the reference's check D^{l1} (x) D^{l2} = c ((+)_l D^l) c^H
within 1e-10; derivative
coefficients within 1e-13 (relative, FP64) of F^l (u_i^l)^T with the host matrices, and
1e-6 for the FP32-data plans; the derivative on points within 1e-7 (relative) of a central
difference of the point evaluation with step 1e-5.
"""
import numpy as np
import pytest

from conftest import rel_err, so3_coeffs

pytestmark = pytest.mark.gpu

PAIRS = [(0, 0), (1, 2), (3, 3), (5, 2), (7, 10), (9, 7)]


@pytest.mark.parametrize("l1,l2", PAIRS)
def test_clebsch_gordan_complex_matches_host(gblib, l1, l2):
    from fftso3_gb300.clebsch_gordan import Clebsch_Gordon_complex
    gpu, host = Clebsch_Gordon_complex(), Clebsch_Gordon_complex()
    gpu.compute(l1, l2)
    host.compute_host(l1, l2)
    assert np.abs(gpu.C - host.C).max() <= 1e-12
    n = gpu.C.shape[0]
    assert np.abs(gpu.C.T @ gpu.C - np.eye(n)).max() <= 1e-11  # orthogonal


@pytest.mark.parametrize("l1,l2", PAIRS)
def test_clebsch_gordan_real_matches_host(gblib, l1, l2):
    from fftso3_gb300.clebsch_gordan import Clebsch_Gordon_real
    gpu, host = Clebsch_Gordon_real(), Clebsch_Gordon_real()
    gpu.compute(l1, l2)
    host.compute_host(l1, l2)
    assert np.abs(gpu.c - host.c).max() <= 1e-12


def test_clebsch_gordan_large_pair_within_recursion_error(gblib):
    """(20, 15): GPU and host run the reference's recursion with different roundings (FMA contraction);
    they agree to the recursion's own error there."""
    from fftso3_gb300.clebsch_gordan import Clebsch_Gordon_complex
    gpu, host = Clebsch_Gordon_complex(), Clebsch_Gordon_complex()
    gpu.compute(20, 15)
    host.compute_host(20, 15)
    assert np.abs(gpu.C - host.C).max() <= 1e-6


def test_clebsch_gordan_reference_check(gblib):
    """The reference's check_Clebsch_Gordon identity with the GPU coefficients (l1, l2) = (3, 5)."""
    import fftso3_gb300 as fg
    assert fg.FFTSO3_real(8, recursion="stable").check_Clebsch_Gordon(3, 5, rng=1) <= 1e-10


def _host_derivative(kind, F, L, axis):
    import fftso3_gb300 as fg
    obj = fg.FFTSO3_complex(L) if kind == "complex" else fg.FFTSO3_real(L)
    u = obj.deriv_wigner_D() if kind == "complex" else obj.deriv_real_harmonics()
    out = []
    for l in range(L + 1):
        W = 2 * l + 1
        o = l * (4 * l * l - 1) // 3
        Fl = F[o:o + W * W].reshape(W, W, order="F")
        out.append((Fl @ u[axis][l].T).ravel(order="F"))
    return np.concatenate(out)


@pytest.mark.parametrize("kind", ["complex", "real"])
@pytest.mark.parametrize("precision", ["fp64", "tc_bf16x3"])
def test_derivative_matches_host_matrices(gblib, kind, precision):
    import torch
    L, b = 12, 3
    cplx = kind == "complex"
    k = gblib.SO3_COMPLEX if cplx else gblib.SO3_REAL
    Fs = [so3_coeffs(L, seed=50 + i, complex_=cplx) for i in range(b)]
    p = gblib.Plan(k, L, b, precision, "stable")
    dt = {("fp64", True): torch.complex128, ("fp64", False): torch.float64,
          ("tc_bf16x3", True): torch.complex64, ("tc_bf16x3", False): torch.float32}[(precision, cplx)]
    c = torch.from_numpy(np.concatenate(Fs)).to(device="cuda", dtype=dt)
    out = torch.empty_like(c)
    s = torch.cuda.current_stream().cuda_stream
    tol = 1e-13 if precision == "fp64" else 1e-6
    for axis in (1, 2, 3):
        p.derivative(c.data_ptr(), axis, out.data_ptr(), s)
        torch.cuda.synchronize()
        got = out.cpu().numpy().astype(np.complex128 if cplx else np.float64).reshape(b, -1)
        for i in range(b):
            assert rel_err(got[i], _host_derivative(kind, Fs[i], L, axis)) <= tol, (axis, i)
    with pytest.raises(gblib.FFTSO3Error):
        p.derivative(c.data_ptr(), 4, out.data_ptr(), s)
    with pytest.raises(gblib.FFTSO3Error):
        p.derivative(c.data_ptr(), 1, c.data_ptr(), s)


@pytest.mark.parametrize("kind", ["complex", "real"])
def test_derivative_is_the_directional_derivative(gblib, kind):
    """f_i(R) from the derivative's coefficients against (f(R exp(h e_i)) - f(R exp(-h e_i))) / 2h."""
    import fftso3_gb300 as fg
    from fftso3_gb300.rotation import euler323_to_R, expm_SO3
    L = 10
    cplx = kind == "complex"
    obj = fg.FFTSO3_complex(L, recursion="stable") if cplx else fg.FFTSO3_real(L, recursion="stable")
    M = fg.FFTSO3_matrix_complex if cplx else fg.FFTSO3_matrix_real
    F = M(L, data=so3_coeffs(L, seed=77, complex_=cplx))
    rng = np.random.default_rng(3)
    h = 1e-5
    for _ in range(4):
        R = euler323_to_R(rng.uniform(-np.pi, np.pi), rng.uniform(0.2, 2.9), rng.uniform(-np.pi, np.pi))
        for axis in (1, 2, 3):
            Fi = obj.derivative(F, axis)
            e = np.zeros(3)
            e[axis - 1] = h
            fd = (obj.inverse_transform(F, R @ expm_SO3(e)) - obj.inverse_transform(F, R @ expm_SO3(-e))) / (2 * h)
            got = obj.inverse_transform(Fi, R)
            assert abs(got - fd) <= 1e-7 * max(1.0, abs(fd)), (axis, got, fd)
