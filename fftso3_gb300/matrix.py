"""Coefficient containers with the indexing of fdcl::FFTSO3_matrix / fdcl::FFTS2_matrix.

``FFTSO3_matrix`` mirrors include/fdcl_FFTSO3_matrix.hpp:44-91: F(l,m,n) reads
one coefficient, F[l] is the (2l+1)x(2l+1) block M[l](m+l, n+l).  The storage
is one packed vector -- the per-l column-major blocks end to end, offset
l(4l^2-1)/3 -- which is exactly the device layout of the C ABI, so a whole
container moves to and from the GPU in one copy.  F[l] is a Fortran-ordered
numpy view into that vector (writes go through).

``FFTS2_matrix`` mirrors include/fdcl_FFTS2_matrix.hpp:40-86: F(l,m), F[l] the
length-(2l+1) vector, packed at l^2 + m + l.
"""
from __future__ import annotations

import numpy as np


def so3_ncoeff(l_max: int) -> int:
    B = l_max + 1
    return B * (4 * B * B - 1) // 3


def so3_offset(l: int) -> int:
    return l * (4 * l * l - 1) // 3


def so3_index(l: int, m: int, n: int) -> int:
    return so3_offset(l) + (m + l) + (n + l) * (2 * l + 1)


def s2_ncoeff(l_max: int) -> int:
    return (l_max + 1) ** 2


def s2_index(l: int, m: int) -> int:
    return l * l + m + l


class _MatrixBase:
    _dtype = np.complex128

    def __init__(self, l_max: int | None = None, data: np.ndarray | None = None):
        self.l_max = -1
        self.M = np.zeros(0, dtype=self._dtype)
        if data is not None:
            if l_max is None:
                raise ValueError("l_max is required with data")
            self.l_max = int(l_max)
            data = np.asarray(data, dtype=self._dtype).reshape(-1)
            if data.size != self._ncoeff(self.l_max):
                raise ValueError(f"data has {data.size} entries, expected {self._ncoeff(self.l_max)}")
            self.M = data
        elif l_max is not None:
            self.init(l_max)

    # -- reference API
    def init(self, l_max: int) -> None:
        if l_max < 0:
            raise ValueError("l_max must be >= 0")
        self.l_max = int(l_max)
        self.M = np.zeros(self._ncoeff(self.l_max), dtype=self._dtype)

    def setZero(self) -> None:
        self.M[:] = 0

    def setRandom(self, rng: np.random.Generator | None = None) -> None:
        """Uniform entries in [-1, 1] (real and imaginary parts), as Eigen's setRandom."""
        rng = rng if rng is not None else np.random.default_rng()
        if np.iscomplexobj(self.M):
            self.M[:] = rng.uniform(-1, 1, self.M.size) + 1j * rng.uniform(-1, 1, self.M.size)
        else:
            self.M[:] = rng.uniform(-1, 1, self.M.size)

    def norm(self) -> float:
        """sum_l ||F^l|| (fdcl_FFTSO3_matrix.cpp:173-181)."""
        tot = 0.0
        for l in range(self.l_max + 1):
            a, b = self._block(l)
            tot += float(np.sqrt(np.sum(np.abs(self.M[a:b]) ** 2)))
        return tot

    def _check_l(self, l: int) -> None:
        if not (0 <= l <= self.l_max):
            raise IndexError(f"l={l} outside [0, {self.l_max}]")

    def __add__(self, other):
        return self._binop(other, np.add)

    def __sub__(self, other):
        return self._binop(other, np.subtract)

    def __mul__(self, c):
        out_t = _complex_t(self) if np.iscomplexobj(np.asarray(c)) else type(self)
        return out_t(self.l_max, data=(self.M * c).astype(out_t._dtype))

    __rmul__ = __mul__

    def _binop(self, other, op):
        if self.l_max != other.l_max:
            raise ValueError("l_max mismatch")
        cplx = np.iscomplexobj(self.M) or np.iscomplexobj(other.M)
        out_t = _complex_t(self) if cplx else type(self)
        return out_t(self.l_max, data=op(self.M, other.M).astype(out_t._dtype))

    def real(self):
        return _real_t(self)(self.l_max, data=np.ascontiguousarray(self.M.real).astype(np.float64))

    def copy(self):
        return type(self)(self.l_max, data=self.M.copy())

    def __str__(self) -> str:
        parts = []
        for l in range(self.l_max + 1):
            parts.append(f"l={l}\n{self[l]}\n")
        return "\n".join(parts)


class FFTSO3_matrix_complex(_MatrixBase):
    _dtype = np.complex128

    @staticmethod
    def _ncoeff(l_max):
        return so3_ncoeff(l_max)

    def _block(self, l):
        return so3_offset(l), so3_offset(l + 1)

    def _check(self, l, m, n):
        self._check_l(l)
        if min(m, n) < -l or max(m, n) > l:
            raise IndexError(f"(m,n)=({m},{n}) outside [-{l},{l}]")

    def __call__(self, l: int, m: int, n: int):
        self._check(l, m, n)
        return self.M[so3_index(l, m, n)]

    def __getitem__(self, key):
        if isinstance(key, tuple):
            l, m, n = key
            return self(l, m, n)
        self._check_l(key)
        a, b = self._block(key)
        w = 2 * key + 1
        return self.M[a:b].reshape((w, w), order="F")

    def __setitem__(self, key, value):
        if isinstance(key, tuple):
            l, m, n = key
            self._check(l, m, n)
            self.M[so3_index(l, m, n)] = value
        else:
            self[key][...] = value


class FFTSO3_matrix_real(FFTSO3_matrix_complex):
    _dtype = np.float64


class FFTS2_matrix_complex(_MatrixBase):
    _dtype = np.complex128

    @staticmethod
    def _ncoeff(l_max):
        return s2_ncoeff(l_max)

    def _block(self, l):
        return l * l, (l + 1) * (l + 1)

    def _check(self, l, m):
        self._check_l(l)
        if not (-l <= m <= l):
            raise IndexError(f"m={m} outside [-{l},{l}]")

    def __call__(self, l: int, m: int):
        self._check(l, m)
        return self.M[s2_index(l, m)]

    def __getitem__(self, key):
        if isinstance(key, tuple):
            l, m = key
            return self(l, m)
        self._check_l(key)
        a, b = self._block(key)
        return self.M[a:b]

    def __setitem__(self, key, value):
        if isinstance(key, tuple):
            l, m = key
            self._check(l, m)
            self.M[s2_index(l, m)] = value
        else:
            self[key][...] = value


class FFTS2_matrix_real(FFTS2_matrix_complex):
    _dtype = np.float64


def _complex_t(x):
    return FFTSO3_matrix_complex if isinstance(x, FFTSO3_matrix_complex) else FFTS2_matrix_complex


def _real_t(x):
    return FFTSO3_matrix_real if isinstance(x, FFTSO3_matrix_complex) else FFTS2_matrix_real
