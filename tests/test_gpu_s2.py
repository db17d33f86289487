"""S^2 parity of the CUDA library against the oracle (GPU).  Tolerance 1e-12
relative for the FP64 path."""
import numpy as np
import pytest

from conftest import rel_err, s2_coeffs

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _run(torch, plan, x, direction, complex_):
    dt = torch.complex128 if complex_ else torch.float64
    a = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    n = plan.batch * (plan.coeff_elems if direction == "fwd" else plan.grid_elems)
    out = torch.empty(n, dtype=dt, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    if direction == "fwd":
        plan.forward(a.data_ptr(), out.data_ptr(), s)
    else:
        plan.inverse(a.data_ptr(), out.data_ptr(), s)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("L", [0, 1, 4, 16, 96, 127])
def test_s2_complex_matches_oracle(gblib, oracle, torch_cuda, L):
    N = 2 * (L + 1)
    F = s2_coeffs(L, seed=L)
    g_ref = oracle.s2_inverse_complex_grid(L, F)
    p = gblib.Plan(gblib.S2_COMPLEX, L)
    g = _run(torch_cuda, p, F, "inv", True).reshape(N, N)
    assert rel_err(g, g_ref) < TOL
    G_ref = oracle.s2_forward_complex(L, g_ref)
    G = _run(torch_cuda, p, g_ref, "fwd", True)
    assert rel_err(G, G_ref) < TOL
    assert rel_err(G, F) < 1e-12


@pytest.mark.parametrize("L", [0, 1, 4, 16, 127])
def test_s2_real_matches_oracle(gblib, oracle, torch_cuda, L):
    N = 2 * (L + 1)
    F = s2_coeffs(L, seed=50 + L, complex_=False)
    g_ref = oracle.s2_inverse_real_grid(L, F)
    p = gblib.Plan(gblib.S2_REAL, L)
    g = _run(torch_cuda, p, F, "inv", False).reshape(N, N)
    assert rel_err(g, g_ref) < TOL
    G_ref = oracle.s2_forward_real(L, g_ref)
    G = _run(torch_cuda, p, g_ref, "fwd", False)
    assert rel_err(G, G_ref) < TOL
    assert rel_err(G, F) < 1e-12


def test_s2_real_l511_batch_roundtrip(gblib, torch_cuda):
    """The S^2 batching workload's shape (1024 x 1024 grid, l_max = 511) at a
    small batch: round trip through the grid returns the coefficients."""
    L, b = 511, 4
    F = np.concatenate([s2_coeffs(L, seed=70 + i, complex_=False) for i in range(b)])
    p = gblib.Plan(gblib.S2_REAL, L, b)
    g = _run(torch_cuda, p, F, "inv", False)
    G = _run(torch_cuda, p, g, "fwd", False)
    assert rel_err(G, F) < 1e-11


def test_s2_point_evaluation(gblib, oracle):
    import fftso3_gb300 as fg
    L = 20
    rng = np.random.default_rng(2)
    pts = np.column_stack([rng.uniform(0.01, np.pi - 0.01, 25), rng.uniform(0, 2 * np.pi, 25)])
    T = fg.FFTS2_complex(L)
    F = fg.FFTS2_matrix_complex(L, data=s2_coeffs(L, 3))
    got = T.inverse_points(F, pts)
    want = np.array([oracle.s2_inverse_complex_point(L, F.M, *p) for p in pts])
    assert rel_err(got, want) < 1e-12
    Tr = fg.FFTS2_real(L)
    Fr = fg.FFTS2_matrix_real(L, data=s2_coeffs(L, 4, complex_=False))
    got = np.array([Tr.inverse_transform(Fr, *p) for p in pts])
    want = np.array([oracle.s2_inverse_real_point(L, Fr.M, *p) for p in pts])
    assert rel_err(got, want) < 1e-12


def test_s2_point_evaluation_partial_warp_many_parts(gblib, oracle):
    """S^2 point evaluation at l_max = 511 (the S^2 batching size) with a partial last warp (70
    points: three batches of 32) and the orders split into many parts, points near both poles
    (where the reference's seed underflows at high m), and a one-point call."""
    import fftso3_gb300 as fg
    L = 511
    rng = np.random.default_rng(5)
    pts = np.column_stack([rng.uniform(0.0, np.pi, 70), rng.uniform(0, 2 * np.pi, 70)])
    pts[0, 0], pts[1, 0] = 1e-3, np.pi - 1e-3
    T = fg.FFTS2_complex(L)
    F = fg.FFTS2_matrix_complex(L, data=s2_coeffs(L, 6))
    got = T.inverse_points(F, pts)
    want = np.array([oracle.s2_inverse_complex_point(L, F.M, *p) for p in pts])
    assert rel_err(got, want) < 1e-12
    one = T.inverse_points(F, pts[7:8])
    assert abs(one[0] - want[7]) < 1e-12 * abs(want[7])


def test_s2_python_api_roundtrip(gblib):
    import fftso3_gb300 as fg
    assert fg.FFTS2_complex(5).check_transform(np.random.default_rng(0)) < 1e-10
    assert fg.FFTS2_real(5).check_transform(np.random.default_rng(1)) < 1e-10
