"""Clebsch-Gordan coefficients of SO(3) harmonics (fdcl::Clebsch_Gordon_complex / _real,
include/fdcl_Clebsch_Gordon.hpp, src/fdcl_Clebsch_Gordon.cpp).

For fixed (l1, l2) the coefficients form one orthogonal matrix C of size
(2 l1 + 1)(2 l2 + 1): row (l1 + m1)(2 l2 + 1) + l2 + m2 for the product basis,
column l^2 - (l2 - l1)^2 + l + m for the coupled basis (l from |l1 - l2|), the
layout and (row, col) formulas of src/fdcl_Clebsch_Gordon.cpp:18-26, so that
    D^{l1} (x) D^{l2} = C (+)_l D^l C^T.
Each column (l, m) solves the three-term relation in m1 that the total angular
momentum eigen-equation gives (the method of the reference's compute_sub,
src/fdcl_Clebsch_Gordon.cpp:41-84, after Straub 2014): started from the largest
m1 and normalised, with the coefficient of the largest m1 positive (the
reference's phase).  The real-harmonic coefficients are
    c = conj(T^{l1} (x) T^{l2}) C ((+)_l T^l)^T,
T = matrix2rsph (src/fdcl_Clebsch_Gordon.cpp:100-120, :179-209), so that
    U^{l1} (x) U^{l2} = c (+)_l U^l c^H.
compute() runs on the GPU (fftso3_clebsch_gordan: one thread per column of C, one
per entry of c); compute_host() is the same recursion in numpy, kept as the CPU
check of the tests.
"""
from __future__ import annotations

import numpy as np

from .transforms import _rsph


class Clebsch_Gordon_complex:
    """C^{l,m}_{l1,m1,l2,m2} for complex harmonics (Wigner D)."""

    def __init__(self, l1: int | None = None, l2: int | None = None):
        self.l1 = self.l2 = -1
        self.C = np.zeros((0, 0))
        if l1 is not None:
            self.init(l1, l2)

    def init(self, l1: int, l2: int) -> None:
        if l1 < 0 or l2 < 0:
            raise ValueError("l1, l2 must be >= 0")
        self.l1, self.l2 = int(l1), int(l2)
        n = (2 * l1 + 1) * (2 * l2 + 1)
        self.C = np.zeros((n, n))

    def row(self, l, m, l1, m1, l2, m2) -> int:
        return (l1 + m1) * (2 * l2 + 1) + l2 + m2

    def col(self, l, m, l1, m1, l2, m2) -> int:
        return l * l - (l2 - l1) * (l2 - l1) + l + m

    def _check(self, l, m, l1, m1, l2, m2) -> None:
        if (l1, l2) != (self.l1, self.l2):
            raise ValueError(f"coefficients computed for (l1, l2) = ({self.l1}, {self.l2})")
        if not (abs(l1 - l2) <= l <= l1 + l2 and -l <= m <= l and -l1 <= m1 <= l1 and -l2 <= m2 <= l2):
            raise ValueError("index out of range")

    def __call__(self, l, m, l1, m1, l2, m2):
        self._check(l, m, l1, m1, l2, m2)
        return self.C[self.row(l, m, l1, m1, l2, m2), self.col(l, m, l1, m1, l2, m2)]

    def compute(self, l1: int, l2: int) -> None:
        """All coefficients of (l1, l2), on the GPU."""
        from . import _lib

        self.init(l1, l2)
        self.C = _lib.clebsch_gordan(l1, l2, real=False)

    def compute_host(self, l1: int, l2: int) -> None:
        """The same coefficients with the recursion in numpy (the CPU check)."""
        self.init(l1, l2)
        for l in range(abs(l1 - l2), l1 + l2 + 1):
            for m in range(-l, l + 1):
                self._column(l, m)

    def _column(self, l: int, m: int) -> None:
        l1, l2 = self.l1, self.l2
        lo, hi = max(-l1, m - l2), min(l1, m + l2)
        if lo > hi:
            return
        a1, a2, al = l1 * (l1 + 1.0), l2 * (l2 + 1.0), l * (l + 1.0)

        def diag(m1):
            return a1 + a2 + 2.0 * m1 * (m - m1) - al

        def off(m1):  # coupling of m1 and m1 - 1
            m2 = m - m1
            return np.sqrt((a1 - m1 * (m1 - 1.0)) * (a2 - m2 * (m2 + 1.0)))

        n = hi - lo + 1
        c = np.zeros(n + 1)  # c[i] for m1 = lo + i; c[n] = 0 above the range
        c[n - 1] = 1.0
        for i in range(n - 1, 0, -1):
            m1 = lo + i
            c[i - 1] = -(diag(m1) * c[i] + off(m1 + 1) * c[i + 1]) / off(m1)
        c = c[:n] / np.linalg.norm(c[:n])
        if c[n - 1] < 0:
            c = -c
        for i in range(n):
            m1 = lo + i
            self.C[self.row(l, m, l1, m1, l2, m - m1), self.col(l, m, l1, m1, l2, m - m1)] = c[i]

    @staticmethod
    def matrix2rsph(L: int) -> list:
        """[T^0, ..., T^L] (src/fdcl_Clebsch_Gordon.cpp:100-120)."""
        return [_rsph(l) for l in range(L + 1)]


class Clebsch_Gordon_real(Clebsch_Gordon_complex):
    """c^{l,m}_{l1,m1,l2,m2} for real harmonics (complex in general)."""

    def init(self, l1: int, l2: int) -> None:
        super().init(l1, l2)
        self.c = np.zeros(self.C.shape, complex)

    def __call__(self, l, m, l1, m1, l2, m2):
        self._check(l, m, l1, m1, l2, m2)
        return self.c[self.row(l, m, l1, m1, l2, m2), self.col(l, m, l1, m1, l2, m2)]

    def compute(self, l1: int, l2: int) -> None:
        """All coefficients of (l1, l2), complex and real harmonics, on the GPU."""
        from . import _lib

        super().compute(l1, l2)
        self.c = _lib.clebsch_gordan(l1, l2, real=True)

    def compute_host(self, l1: int, l2: int) -> None:
        super().compute_host(l1, l2)
        T1, T2 = _rsph(l1), _rsph(l2)
        T12 = np.kron(T1, T2)
        n = self.C.shape[0]
        OT = np.zeros((n, n), complex)
        i = 0
        for l in range(abs(l1 - l2), l1 + l2 + 1):
            OT[i:i + 2 * l + 1, i:i + 2 * l + 1] = _rsph(l)
            i += 2 * l + 1
        self.c = np.conj(T12) @ self.C @ OT.T
