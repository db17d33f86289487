"""ctypes front end of the compiled reference (test infrastructure only).

``oracle/ref.mk`` compiles the reference's own transform sources, unmodified,
against the Eigen-API subset in ``oracle/ref_shim/`` into
``oracle/_ref/libfdcl_ref.so``, with the C entry points of ``ref_capi.cpp``.
It needs the reference's source tree, so it exists only where that tree does;
``available()`` says whether it could be built.  Its outputs pin the restated
oracle (``oracle.py``) and, through the fixtures that
``tests/golden/make_ref_fixtures.py`` writes, the CUDA library.  The product
never imports this module.

Array conventions are the oracle's (``oracle.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libfdcl_ref.so")
_MK = os.path.join(_HERE, "ref.mk")
_lib = None
_dp = ctypes.POINTER(ctypes.c_double)


def build() -> bool:
    """Build the compiled reference when the reference tree is present; False when it is not (or the build
    fails, e.g. on a host without the sources)."""
    if subprocess.run(["make", "-s", "-f", _MK, "check"], capture_output=True).returncode != 0:
        return os.path.exists(_LIB_PATH)
    r = subprocess.run(["make", "-s", "-j8", "-f", _MK], capture_output=True, text=True)
    return r.returncode == 0 and os.path.exists(_LIB_PATH)


def available() -> bool:
    try:
        lib()
        return True
    except OSError:
        return False


def lib():
    global _lib
    if _lib is None:
        if not build():
            raise OSError("compiled reference unavailable: the reference's sources are not on this host")
        L = ctypes.CDLL(_LIB_PATH)
        i, d = ctypes.c_int, ctypes.c_double
        sig = {
            "ref_so3_forward_complex": [i, _dp, _dp],
            "ref_so3_forward_real": [i, _dp, _dp],
            "ref_so3_inverse_complex_point": [i, _dp, d, d, d, _dp],
            "ref_so3_inverse_real_point": [i, _dp, d, d, d, _dp],
            "ref_wigner_d": [i, d, _dp],
            "ref_so3_real_harmonics": [i, d, d, d, _dp],
            "ref_s2_forward_complex": [i, _dp, _dp],
            "ref_s2_forward_real": [i, _dp, _dp],
            "ref_s2_inverse_complex_point": [i, _dp, d, d, _dp],
            "ref_s2_inverse_real_point": [i, _dp, d, d, _dp],
            "ref_clebsch_gordan_complex": [i, i, _dp, ctypes.POINTER(ctypes.c_int)],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _ok(rc: int) -> None:
    if rc != 0:
        raise RuntimeError("the compiled reference raised an exception")


def so3_ncoeff(L: int) -> int:
    return (L + 1) * (4 * (L + 1) ** 2 - 1) // 3


def so3_forward_complex(L: int, grid: np.ndarray) -> np.ndarray:
    """fdcl::FFTSO3_complex::forward_transform of the samples grid[k, j1, j2]."""
    g = np.ascontiguousarray(grid, dtype=np.complex128)
    out = np.zeros(so3_ncoeff(L), np.complex128)
    _ok(lib().ref_so3_forward_complex(L, _p(g), _p(out)))
    return out


def so3_forward_real(L: int, grid: np.ndarray) -> np.ndarray:
    """fdcl::FFTSO3_real::forward_transform of the real samples grid[k, j1, j2]."""
    g = np.ascontiguousarray(grid, dtype=np.float64)
    out = np.zeros(so3_ncoeff(L))
    _ok(lib().ref_so3_forward_real(L, _p(g), _p(out)))
    return out


def so3_inverse_complex_point(L: int, F: np.ndarray, a: float, b: float, c: float) -> complex:
    f = np.ascontiguousarray(F, dtype=np.complex128)
    out = np.zeros(2)
    _ok(lib().ref_so3_inverse_complex_point(L, _p(f), a, b, c, _p(out)))
    return complex(out[0], out[1])


def so3_inverse_real_point(L: int, F: np.ndarray, a: float, b: float, c: float) -> float:
    f = np.ascontiguousarray(F, dtype=np.float64)
    out = np.zeros(1)
    _ok(lib().ref_so3_inverse_real_point(L, _p(f), a, b, c, _p(out)))
    return float(out[0])


def wigner_d(beta: float, L: int) -> np.ndarray:
    out = np.zeros(so3_ncoeff(L))
    _ok(lib().ref_wigner_d(L, beta, _p(out)))
    return out


def so3_real_harmonics(L: int, a: float, b: float, c: float) -> np.ndarray:
    out = np.zeros(so3_ncoeff(L))
    _ok(lib().ref_so3_real_harmonics(L, a, b, c, _p(out)))
    return out


def s2_forward_complex(L: int, grid: np.ndarray) -> np.ndarray:
    g = np.ascontiguousarray(grid, dtype=np.complex128)
    out = np.zeros((L + 1) ** 2, np.complex128)
    _ok(lib().ref_s2_forward_complex(L, _p(g), _p(out)))
    return out


def s2_forward_real(L: int, grid: np.ndarray) -> np.ndarray:
    g = np.ascontiguousarray(grid, dtype=np.float64)
    out = np.zeros((L + 1) ** 2)
    _ok(lib().ref_s2_forward_real(L, _p(g), _p(out)))
    return out


def s2_inverse_complex_point(L: int, F: np.ndarray, theta: float, phi: float) -> complex:
    f = np.ascontiguousarray(F, dtype=np.complex128)
    out = np.zeros(2)
    _ok(lib().ref_s2_inverse_complex_point(L, _p(f), theta, phi, _p(out)))
    return complex(out[0], out[1])


def s2_inverse_real_point(L: int, F: np.ndarray, theta: float, phi: float) -> float:
    f = np.ascontiguousarray(F, dtype=np.float64)
    out = np.zeros(1)
    _ok(lib().ref_s2_inverse_real_point(L, _p(f), theta, phi, _p(out)))
    return float(out[0])


def clebsch_gordan_complex(l1: int, l2: int) -> np.ndarray:
    """The coefficient matrix C of fdcl::Clebsch_Gordon_complex::compute(l1, l2)."""
    n = ctypes.c_int()
    _ok(lib().ref_clebsch_gordan_complex(l1, l2, None, ctypes.byref(n)))
    C = np.zeros(n.value * n.value)
    _ok(lib().ref_clebsch_gordan_complex(l1, l2, _p(C), ctypes.byref(n)))
    return C.reshape(n.value, n.value, order="F")
