"""Pins the oracle to the reference's own code, compiled (no GPU).

oracle/ref.mk compiles the reference's transform sources unmodified against a
self-written Eigen-API subset (oracle/ref_shim/), and oracle/ref.py calls them.

* Fixture tests (any host): tests/golden/reference_compiled.npz holds what the
  compiled reference returned (tests/golden/make_ref_fixtures.py) for inputs
  the oracle rebuilds from seeded coefficients: l_max = 16 in full and
  l_max = 127 at 2048 sampled coefficients plus the per-degree norms.  The
  oracle must agree within 1e-12 relative (measured ~3e-16).
* Live tests (only where the reference's sources are present, else skipped):
  the compiled reference against the oracle on fresh inputs -- forward
  transforms within 1e-13 relative, point inverses within 1e-13, wigner_d and
  the real harmonics bit for bit (both built without FMA contraction), the
  Clebsch-Gordan matrices within 1e-12 of the host port.
"""
import os

import numpy as np
import pytest

from conftest import rel_err, s2_coeffs, so3_coeffs

FIX = os.path.join(os.path.dirname(__file__), "golden", "reference_compiled.npz")
SEEDS = {"so3c": 1601, "so3r": 1602, "s2c": 1603, "s2r": 1604, "l127c": 12701, "l127r": 12702}


@pytest.fixture(scope="module")
def fx():
    return np.load(FIX)


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as R
    if not R.available():
        pytest.skip("the reference's sources are not on this host")
    return R


def _l16_inputs(oracle):
    L, N = 16, 34
    F = so3_coeffs(L, SEEDS["so3c"])
    Fr = so3_coeffs(L, SEEDS["so3r"], complex_=False)
    S = s2_coeffs(L, SEEDS["s2c"])
    Sr = s2_coeffs(L, SEEDS["s2r"], complex_=False)
    return L, N, F, Fr, S, Sr


def test_fixture_l16_forward_transforms(oracle, fx):
    L, N, F, Fr, S, Sr = _l16_inputs(oracle)
    got = {
        "l16_so3_complex": oracle.so3_forward_complex(L, oracle.so3_inverse_complex_grid(L, F).reshape(N, N, N)),
        "l16_so3_real": oracle.so3_forward_real(L, oracle.so3_inverse_real_grid(L, Fr).reshape(N, N, N)),
        "l16_s2_complex": oracle.s2_forward_complex(L, oracle.s2_inverse_complex_grid(L, S).reshape(N, N)),
        "l16_s2_real": oracle.s2_forward_real(L, oracle.s2_inverse_real_grid(L, Sr).reshape(N, N)),
    }
    for k, v in got.items():
        assert rel_err(v, fx[k]) <= 1e-12, k
    # and the reference's forward recovers the synthesised coefficients (l_max = 16: no recursion loss)
    assert rel_err(fx["l16_so3_complex"], F) <= 1e-13
    assert rel_err(fx["l16_so3_real"], Fr) <= 1e-13


def test_fixture_l16_points_and_wigner_d(oracle, fx):
    L, N, F, Fr, S, Sr = _l16_inputs(oracle)
    for i, (a, b, c) in enumerate(fx["l16_points"]):
        assert abs(oracle.so3_inverse_complex_point(L, F, a, b, c) - fx["l16_so3_complex_points"][i]) <= 1e-12
        assert abs(oracle.so3_inverse_real_point(L, Fr, a, b, c) - fx["l16_so3_real_points"][i]) <= 1e-12
        assert abs(oracle.s2_inverse_complex_point(L, S, b, a) - fx["l16_s2_complex_points"][i]) <= 1e-12
        assert abs(oracle.s2_inverse_real_point(L, Sr, b, a) - fx["l16_s2_real_points"][i]) <= 1e-12
    assert np.abs(oracle.wigner_d(float(fx["l16_wigner_d_beta"]), L) - fx["l16_wigner_d"]).max() <= 1e-14


@pytest.mark.parametrize("kind", ["complex", "real"])
def test_fixture_l127_forward_samples(oracle, fx, kind):
    """The 256^3 case: the reference's own forward at l_max = 127, including its Wigner-d recursion's loss there
    (the recovered coefficients differ from the synthesised ones by ~5e-3 relative), at 2048 sampled places and
    in the per-degree norms."""
    L, N = 127, 256
    cplx = kind == "complex"
    F = so3_coeffs(L, SEEDS["l127c" if cplx else "l127r"], complex_=cplx)
    if cplx:
        G = oracle.so3_forward_complex(L, oracle.so3_inverse_complex_grid(L, F).reshape(N, N, N))
    else:
        G = oracle.so3_forward_real(L, oracle.so3_inverse_real_grid(L, F).reshape(N, N, N))
    idx = fx["l127_index"]
    assert rel_err(G[idx], fx[f"l127_so3_{kind}"]) <= 1e-12
    norms = np.array([np.linalg.norm(G[l * (4 * l * l - 1) // 3:(l + 1) * (4 * (l + 1) ** 2 - 1) // 3])
                      for l in range(L + 1)])
    assert np.abs(norms / fx[f"l127_so3_{kind}_norms"] - 1).max() <= 1e-12


@pytest.mark.parametrize("L", [0, 3, 8, 16])
def test_live_forward_transforms(oracle, ref, L):
    N = 2 * (L + 1)
    F = so3_coeffs(L, 900 + L)
    g = oracle.so3_inverse_complex_grid(L, F).reshape(N, N, N)
    assert rel_err(ref.so3_forward_complex(L, g), oracle.so3_forward_complex(L, g)) <= 1e-13
    Fr = so3_coeffs(L, 910 + L, complex_=False)
    g = oracle.so3_inverse_real_grid(L, Fr).reshape(N, N, N)
    assert rel_err(ref.so3_forward_real(L, g), oracle.so3_forward_real(L, g)) <= 1e-13
    S = s2_coeffs(L, 920 + L)
    g = oracle.s2_inverse_complex_grid(L, S).reshape(N, N)
    assert rel_err(ref.s2_forward_complex(L, g), oracle.s2_forward_complex(L, g)) <= 1e-13
    Sr = s2_coeffs(L, 930 + L, complex_=False)
    g = oracle.s2_inverse_real_grid(L, Sr).reshape(N, N)
    assert rel_err(ref.s2_forward_real(L, g), oracle.s2_forward_real(L, g)) <= 1e-13


def test_live_forward_of_non_bandlimited_samples(oracle, ref):
    """Arbitrary samples (not a synthesis): the aliasing terms must match as well."""
    L, N = 7, 16
    rng = np.random.Generator(np.random.PCG64(5))
    g = rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))
    assert rel_err(ref.so3_forward_complex(L, g), oracle.so3_forward_complex(L, g)) <= 1e-13
    assert rel_err(ref.so3_forward_real(L, g.real), oracle.so3_forward_real(L, g.real)) <= 1e-13


def test_live_point_inverses_wigner_d_and_real_harmonics(oracle, ref):
    L = 12
    rng = np.random.Generator(np.random.PCG64(6))
    F = so3_coeffs(L, 940)
    Fr = so3_coeffs(L, 941, complex_=False)
    S = s2_coeffs(L, 942)
    Sr = s2_coeffs(L, 943, complex_=False)
    for _ in range(6):
        a, c = rng.uniform(-np.pi, np.pi, 2)
        b = rng.uniform(0.01, np.pi - 0.01)
        assert abs(ref.so3_inverse_complex_point(L, F, a, b, c) - oracle.so3_inverse_complex_point(L, F, a, b, c)) <= 1e-13
        assert abs(ref.so3_inverse_real_point(L, Fr, a, b, c) - oracle.so3_inverse_real_point(L, Fr, a, b, c)) <= 1e-13
        assert abs(ref.s2_inverse_complex_point(L, S, b, a) - oracle.s2_inverse_complex_point(L, S, b, a)) <= 1e-13
        assert abs(ref.s2_inverse_real_point(L, Sr, b, a) - oracle.s2_inverse_real_point(L, Sr, b, a)) <= 1e-13
        assert np.array_equal(ref.wigner_d(b, L), oracle.wigner_d(b, L))
        assert np.array_equal(ref.so3_real_harmonics(L, a, b, c), oracle.so3_real_harmonics(L, a, b, c))


@pytest.mark.parametrize("l1,l2", [(0, 0), (1, 2), (3, 3), (5, 2), (7, 10), (9, 7)])
def test_live_clebsch_gordan(ref, l1, l2):
    from fftso3_gb300.clebsch_gordan import Clebsch_Gordon_complex
    h = Clebsch_Gordon_complex()
    h.compute_host(l1, l2)
    C = ref.clebsch_gordan_complex(l1, l2)
    assert C.shape == h.C.shape
    assert np.abs(C - h.C).max() <= 1e-12
