"""numpy front end of the CPU oracle (test infrastructure only).

Loads ``oracle/libfftso3_oracle.so`` (built from ``fftso3_oracle.c`` by the
Makefile next to this file) and exposes the restated reference algorithms on
numpy arrays.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` import this module; the product package never does.

Array conventions (shared with the product):
  SO(3) coefficients: packed complex128/float64 vector, (l,m,n) at
    l(4l^2-1)/3 + (m+l) + (n+l)(2l+1).
  S^2 coefficients: packed vector, (l,m) at l^2 + m + l.
  SO(3) grid: (N, N, N) array indexed [k, j1, j2] = f(alpha_j1, beta_k, gamma_j2).
  S^2 grid:  (N, N) array indexed [k, j] = f(theta_k, phi_j).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libfftso3_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)


def build() -> str:
    """Compile the oracle with its Makefile (no-op when up to date)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "fftso3_oracle.c"))
        ):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        i, d, l_ = ctypes.c_int, ctypes.c_double, ctypes.c_long
        sig = {
            "orc_so3_ncoeff": (l_, [i]),
            "orc_s2_ncoeff": (l_, [i]),
            "orc_beta_k": (d, [i, i]),
            "orc_alpha_j": (d, [i, i]),
            "orc_so3_weights": (None, [i, _dp]),
            "orc_s2_weights": (None, [i, _dp]),
            "orc_wigner_d": (None, [d, i, _dp]),
            "orc_wigner_d_explicit": (None, [d, _dp]),
            "orc_nor_assoc_legendre": (None, [d, i, _dp]),
            "orc_dft": (None, [i, _dp, l_, _dp, l_]),
            "orc_so3_forward_complex": (None, [i, _dp, i, _dp]),
            "orc_so3_forward_real": (None, [i, _dp, _dp]),
            "orc_so3_inverse_complex_point": (None, [i, _dp, d, d, d, _dp]),
            "orc_so3_inverse_real_point": (d, [i, _dp, d, d, d]),
            "orc_so3_real_harmonics": (None, [i, d, d, d, _dp]),
            "orc_so3_inverse_complex_grid": (None, [i, _dp, _dp]),
            "orc_so3_forward_complex_slices": (None, [i, _dp, _dp, i, i]),
            "orc_so3_inverse_complex_slices": (None, [i, _dp, _dp, i, i]),
            "orc_so3_forward_complex_strided": (None, [i, _dp, _dp, i, i, i]),
            "orc_so3_inverse_complex_strided": (None, [i, _dp, _dp, i, i, i]),
            "orc_so3_inverse_real_grid": (None, [i, _dp, _dp]),
            "orc_so3_real_to_complex": (None, [i, _dp, _dp]),
            "orc_s2_forward_complex": (None, [i, _dp, i, _dp]),
            "orc_s2_forward_real": (None, [i, _dp, _dp]),
            "orc_s2_inverse_complex_point": (None, [i, _dp, d, d, _dp]),
            "orc_s2_inverse_real_point": (d, [i, _dp, d, d]),
            "orc_s2_inverse_complex_grid": (None, [i, _dp, _dp]),
            "orc_s2_inverse_real_grid": (None, [i, _dp, _dp]),
            "orc_s2_real_to_complex": (None, [i, _dp, _dp]),
            "orc_num_threads": (i, []),
            "orc_set_num_threads": (None, [i]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(_dp)


def so3_ncoeff(l_max: int) -> int:
    B = l_max + 1
    return B * (4 * B * B - 1) // 3


def s2_ncoeff(l_max: int) -> int:
    return (l_max + 1) ** 2


def so3_index(l: int, m: int, n: int) -> int:
    return l * (4 * l * l - 1) // 3 + (m + l) + (n + l) * (2 * l + 1)


def s2_index(l: int, m: int) -> int:
    return l * l + m + l


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def num_threads() -> int:
    return lib().orc_num_threads()


def beta_k(l_max: int, k: int) -> float:
    return lib().orc_beta_k(l_max + 1, k)


def alpha_j(l_max: int, j: int) -> float:
    return lib().orc_alpha_j(l_max + 1, j)


def so3_weights(l_max: int) -> np.ndarray:
    w = np.zeros(2 * (l_max + 1))
    lib().orc_so3_weights(l_max, _p(w))
    return w


def s2_weights(l_max: int) -> np.ndarray:
    w = np.zeros(2 * (l_max + 1))
    lib().orc_s2_weights(l_max, _p(w))
    return w


def wigner_d(beta: float, l_max: int) -> np.ndarray:
    d = np.zeros(so3_ncoeff(l_max))
    lib().orc_wigner_d(float(beta), l_max, _p(d))
    return d


def wigner_d_explicit(beta: float) -> np.ndarray:
    d = np.zeros(so3_ncoeff(3))
    lib().orc_wigner_d_explicit(float(beta), _p(d))
    return d


def nor_assoc_legendre(x: float, l_max: int) -> np.ndarray:
    nP = np.zeros(s2_ncoeff(l_max))
    lib().orc_nor_assoc_legendre(float(x), l_max, _p(nP))
    return nP


def dft(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.zeros_like(x)
    lib().orc_dft(len(x), _p(x.view(np.float64)), 1, _p(out.view(np.float64)), 1)
    return out


def so3_forward_complex(l_max: int, grid: np.ndarray, is_real: bool = False) -> np.ndarray:
    N = 2 * (l_max + 1)
    g = np.ascontiguousarray(grid, dtype=np.complex128)
    assert g.shape == (N, N, N)
    F = np.zeros(so3_ncoeff(l_max), dtype=np.complex128)
    lib().orc_so3_forward_complex(l_max, _p(g.view(np.float64)), int(bool(is_real)), _p(F.view(np.float64)))
    return F


def so3_forward_real(l_max: int, grid: np.ndarray) -> np.ndarray:
    N = 2 * (l_max + 1)
    g = np.ascontiguousarray(grid, dtype=np.float64)
    assert g.shape == (N, N, N)
    F = np.zeros(so3_ncoeff(l_max))
    lib().orc_so3_forward_real(l_max, _p(g), _p(F))
    return F


def so3_inverse_complex_point(l_max: int, F: np.ndarray, alpha: float, beta: float, gamma: float) -> complex:
    F = np.ascontiguousarray(F, dtype=np.complex128)
    out = np.zeros(2)
    lib().orc_so3_inverse_complex_point(l_max, _p(F.view(np.float64)), alpha, beta, gamma, _p(out))
    return complex(out[0], out[1])


def so3_inverse_real_point(l_max: int, F: np.ndarray, alpha: float, beta: float, gamma: float) -> float:
    F = np.ascontiguousarray(F, dtype=np.float64)
    return lib().orc_so3_inverse_real_point(l_max, _p(F), alpha, beta, gamma)


def so3_real_harmonics(l_max: int, alpha: float, beta: float, gamma: float) -> np.ndarray:
    U = np.zeros(so3_ncoeff(l_max))
    lib().orc_so3_real_harmonics(l_max, alpha, beta, gamma, _p(U))
    return U


def so3_inverse_complex_grid(l_max: int, F: np.ndarray) -> np.ndarray:
    N = 2 * (l_max + 1)
    F = np.ascontiguousarray(F, dtype=np.complex128)
    g = np.zeros((N, N, N), dtype=np.complex128)
    lib().orc_so3_inverse_complex_grid(l_max, _p(F.view(np.float64)), _p(g.view(np.float64)))
    return g


def so3_forward_complex_slices(l_max: int, slab: np.ndarray, k0: int, k1: int) -> np.ndarray:
    """Contribution of the beta slices k0..k1-1 to the complex forward sum
    (slab: (k1-k0, N, N) complex); used for bounded CPU timing samples."""
    N = 2 * (l_max + 1)
    g = np.ascontiguousarray(slab, dtype=np.complex128)
    assert g.shape == (k1 - k0, N, N)
    F = np.zeros(so3_ncoeff(l_max), dtype=np.complex128)
    lib().orc_so3_forward_complex_slices(l_max, _p(g.view(np.float64)), _p(F.view(np.float64)), k0, k1)
    return F


def so3_inverse_complex_slices(l_max: int, F: np.ndarray, k0: int, k1: int) -> np.ndarray:
    """Grid synthesis of the beta slices k0..k1-1 only: (k1-k0, N, N) complex."""
    N = 2 * (l_max + 1)
    F = np.ascontiguousarray(F, dtype=np.complex128)
    g = np.zeros((k1 - k0, N, N), dtype=np.complex128)
    lib().orc_so3_inverse_complex_slices(l_max, _p(F.view(np.float64)), _p(g.view(np.float64)), k0, k1)
    return g


def so3_forward_complex_strided(l_max: int, slab: np.ndarray, k0: int, kstride: int) -> np.ndarray:
    """Contribution of the beta slices k0 + i kstride (slab[i], i < len(slab)) to the complex forward sum;
    CPU timing samples spread over [0, pi)."""
    N = 2 * (l_max + 1)
    g = np.ascontiguousarray(slab, dtype=np.complex128)
    assert g.ndim == 3 and g.shape[1:] == (N, N) and k0 + (g.shape[0] - 1) * kstride < N
    F = np.zeros(so3_ncoeff(l_max), dtype=np.complex128)
    lib().orc_so3_forward_complex_strided(l_max, _p(g.view(np.float64)), _p(F.view(np.float64)), k0, kstride,
                                          g.shape[0])
    return F


def so3_inverse_complex_strided(l_max: int, F: np.ndarray, k0: int, kstride: int, count: int) -> np.ndarray:
    """Grid synthesis of the beta slices k0 + i kstride, i < count: (count, N, N) complex."""
    N = 2 * (l_max + 1)
    assert k0 + (count - 1) * kstride < N
    F = np.ascontiguousarray(F, dtype=np.complex128)
    g = np.zeros((count, N, N), dtype=np.complex128)
    lib().orc_so3_inverse_complex_strided(l_max, _p(F.view(np.float64)), _p(g.view(np.float64)), k0, kstride, count)
    return g


def so3_inverse_real_grid(l_max: int, F: np.ndarray) -> np.ndarray:
    N = 2 * (l_max + 1)
    F = np.ascontiguousarray(F, dtype=np.float64)
    g = np.zeros((N, N, N))
    lib().orc_so3_inverse_real_grid(l_max, _p(F), _p(g))
    return g


def so3_real_to_complex(l_max: int, F: np.ndarray) -> np.ndarray:
    F = np.ascontiguousarray(F, dtype=np.float64)
    Fc = np.zeros(so3_ncoeff(l_max), dtype=np.complex128)
    lib().orc_so3_real_to_complex(l_max, _p(F), _p(Fc.view(np.float64)))
    return Fc


def s2_forward_complex(l_max: int, grid: np.ndarray, is_real: bool = False) -> np.ndarray:
    N = 2 * (l_max + 1)
    g = np.ascontiguousarray(grid, dtype=np.complex128)
    assert g.shape == (N, N)
    F = np.zeros(s2_ncoeff(l_max), dtype=np.complex128)
    lib().orc_s2_forward_complex(l_max, _p(g.view(np.float64)), int(bool(is_real)), _p(F.view(np.float64)))
    return F


def s2_forward_real(l_max: int, grid: np.ndarray) -> np.ndarray:
    N = 2 * (l_max + 1)
    g = np.ascontiguousarray(grid, dtype=np.float64)
    assert g.shape == (N, N)
    F = np.zeros(s2_ncoeff(l_max))
    lib().orc_s2_forward_real(l_max, _p(g), _p(F))
    return F


def s2_inverse_complex_point(l_max: int, F: np.ndarray, theta: float, phi: float) -> complex:
    F = np.ascontiguousarray(F, dtype=np.complex128)
    out = np.zeros(2)
    lib().orc_s2_inverse_complex_point(l_max, _p(F.view(np.float64)), theta, phi, _p(out))
    return complex(out[0], out[1])


def s2_inverse_real_point(l_max: int, F: np.ndarray, theta: float, phi: float) -> float:
    F = np.ascontiguousarray(F, dtype=np.float64)
    return lib().orc_s2_inverse_real_point(l_max, _p(F), theta, phi)


def s2_inverse_complex_grid(l_max: int, F: np.ndarray) -> np.ndarray:
    N = 2 * (l_max + 1)
    F = np.ascontiguousarray(F, dtype=np.complex128)
    g = np.zeros((N, N), dtype=np.complex128)
    lib().orc_s2_inverse_complex_grid(l_max, _p(F.view(np.float64)), _p(g.view(np.float64)))
    return g


def s2_inverse_real_grid(l_max: int, F: np.ndarray) -> np.ndarray:
    N = 2 * (l_max + 1)
    F = np.ascontiguousarray(F, dtype=np.float64)
    g = np.zeros((N, N))
    lib().orc_s2_inverse_real_grid(l_max, _p(F), _p(g))
    return g


def s2_real_to_complex(l_max: int, F: np.ndarray) -> np.ndarray:
    F = np.ascontiguousarray(F, dtype=np.float64)
    Fc = np.zeros(s2_ncoeff(l_max), dtype=np.complex128)
    lib().orc_s2_real_to_complex(l_max, _p(F), _p(Fc.view(np.float64)))
    return Fc


def per_l_norm_sum(F: np.ndarray, l_max: int, kind: str = "so3") -> float:
    """sum_l ||F^l||_Frobenius, the reference's container norm
    (fdcl_FFTSO3_matrix.cpp:173-181, fdcl_FFTS2_matrix.cpp:169-177)."""
    tot = 0.0
    for l in range(l_max + 1):
        if kind == "so3":
            a, b = l * (4 * l * l - 1) // 3, (l + 1) * (4 * (l + 1) ** 2 - 1) // 3
        else:
            a, b = l * l, (l + 1) ** 2
        tot += float(np.sqrt(np.sum(np.abs(F[a:b]) ** 2)))
    return tot
