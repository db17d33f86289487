"""The four transform classes of fdcl-gwu/FFTSO3 on the GB300 library.

``FFTSO3_complex``, ``FFTSO3_real`` (include/fdcl_FFTSO3.hpp:27-308) and
``FFTS2_complex``, ``FFTS2_real`` (include/fdcl_FFTS2.hpp:28-160) with the
reference's method names and argument meanings:

* ``forward_transform(func)`` samples ``func`` on the Euler (or theta, phi)
  grid on the host -- vectorised when ``func`` accepts numpy arrays, point by
  point otherwise, like the reference's OpenMP callback loop
  (fdcl_FFTSO3.cpp:676-685) -- then runs the transform on the GPU.  It also
  accepts the sampled grid itself (an ndarray of the grid's shape).
  A one-argument ``func`` is read as ``f(R)`` on rotation matrices
  (fdcl_FFTSO3.cpp:934-941); for S^2 the two arguments are (theta, phi).
* ``inverse_transform(F, alpha, beta, gamma)`` / ``(F, R)`` evaluates the series
  at a point on the GPU (fdcl_FFTSO3.cpp:498-531, :1141-1167); like the
  reference it re-initialises the object to ``F.l_max``.
* ``inverse_grid(F)`` synthesises the whole grid (the GPU grid inverse).

Every transform runs in the CUDA library; nothing here computes a transform
on the CPU.
"""
from __future__ import annotations

import ctypes
import inspect

import numpy as np

from . import _lib
from .matrix import (FFTS2_matrix_complex, FFTS2_matrix_real, FFTSO3_matrix_complex, FFTSO3_matrix_real,
                     so3_ncoeff, s2_ncoeff)
from .rotation import R_to_euler323, euler323_to_R


def beta_k(l_max: int, k) -> np.ndarray:
    """beta_k = (2k+1) pi / (4B) (fdcl_FFTSO3.cpp:578-581)."""
    B = l_max + 1
    return (2.0 * np.asarray(k, float) + 1.0) * np.pi / 4.0 / B


def alpha_j(l_max: int, j) -> np.ndarray:
    """alpha_j = gamma_j = j pi / B (fdcl_FFTSO3.cpp:583-591)."""
    return np.asarray(j, float) * np.pi / (l_max + 1)


def _n_params(func) -> int:
    try:
        sig = inspect.signature(func)
    except (TypeError, ValueError):
        return -1
    n = 0
    for p in sig.parameters.values():
        if p.kind in (p.VAR_POSITIONAL,):
            return -1
        if p.default is p.empty and p.kind in (p.POSITIONAL_ONLY, p.POSITIONAL_OR_KEYWORD):
            n += 1
    return n


def _sample(func, args, shape, dtype):
    """Evaluate func on broadcast grid arrays; vectorised first, else point by point."""
    try:
        v = np.asarray(func(*args))
        if v.shape == shape:
            return v.astype(dtype, copy=False)
    except Exception:
        pass
    flat = [np.asarray(a).reshape(-1) for a in np.broadcast_arrays(*args)]
    out = np.empty(flat[0].size, dtype=dtype)
    for i in range(out.size):
        out[i] = func(*(float(a[i]) for a in flat))
    return out.reshape(shape)


class _Transform:
    _kind = None
    _complex = True
    _so3 = True

    def __init__(self, l_max: int | None = None, *, precision: str = "fp64", recursion: str = "reference",
                 refine: bool = False):
        self.precision = precision
        self.recursion = recursion
        self.refine = refine
        self.check_verbose = False
        self.l_max = -1
        self._plan = None
        if l_max is not None:
            self.init(l_max)

    # -- reference API
    def init(self, l_max: int) -> None:
        if l_max < 0:
            raise ValueError("l_max must be >= 0")
        if l_max != self.l_max:
            self.l_max = int(l_max)
            self.B = self.l_max + 1
            self._plan = None

    @property
    def plan(self) -> _lib.Plan:
        if self._plan is None:
            self._plan = _lib.Plan(self._kind, self.l_max, 1, self.precision, self.recursion,
                                   _lib.FLAG_REFINE if self.refine else 0)
        return self._plan

    @property
    def N(self) -> int:
        return 2 * (self.l_max + 1)

    def grid_shape(self) -> tuple:
        N = self.N
        return (N, N, N) if self._so3 else (N, N)

    def _grid_dtype(self):
        if self.precision == "fp64":
            return np.complex128 if self._complex else np.float64
        return np.complex64 if self._complex else np.float32

    def _coeff_dtype(self):
        return self._grid_dtype()

    def weights(self) -> np.ndarray:
        w = np.zeros(self.N)
        _lib.check(_lib.lib().fftso3_weights(self._kind, self.l_max, w.ctypes.data_as(_lib._dp)))
        return w

    # -- sampling
    def sample(self, func) -> np.ndarray:
        N = self.N
        dt = self._grid_dtype()
        b = beta_k(self.l_max, np.arange(N))
        a = alpha_j(self.l_max, np.arange(N))
        if self._so3:
            K, J1, J2 = np.meshgrid(b, a, a, indexing="ij")
            if _n_params(func) == 1:
                R = euler323_to_R(J1, K, J2)
                try:
                    v = np.asarray(func(R))
                    if v.shape == K.shape:
                        return v.astype(dt, copy=False)
                except Exception:
                    pass
                out = np.empty(K.size, dtype=dt)
                Rf = R.reshape(-1, 3, 3)
                for i in range(out.size):
                    out[i] = func(Rf[i])
                return out.reshape(K.shape)
            return _sample(func, (J1, K, J2), K.shape, dt)
        T, P = np.meshgrid(b, a, indexing="ij")
        return _sample(func, (T, P), T.shape, dt)

    # -- transforms
    def _coeff_container(self, data):
        raise NotImplementedError

    def forward_transform(self, func):
        grid = func if isinstance(func, np.ndarray) else self.sample(func)
        grid = np.ascontiguousarray(grid, dtype=self._grid_dtype())
        if grid.shape != self.grid_shape():
            raise ValueError(f"grid shape {grid.shape}, expected {self.grid_shape()}")
        ncoef = so3_ncoeff(self.l_max) if self._so3 else s2_ncoeff(self.l_max)
        out = np.empty(ncoef, dtype=self._coeff_dtype())
        self.plan.forward_host(grid.ctypes.data, out.ctypes.data)
        return self._coeff_container(out)

    def inverse_grid(self, F) -> np.ndarray:
        """f on the whole sampling grid (the grid form of inverse_transform)."""
        self.init(F.l_max)
        c = np.ascontiguousarray(F.M, dtype=self._coeff_dtype())
        grid = np.empty(self.grid_shape(), dtype=self._grid_dtype())
        self.plan.inverse_host(c.ctypes.data, grid.ctypes.data)
        return grid

    def _points(self, F, pts: np.ndarray) -> np.ndarray:
        import torch

        self.init(F.l_max)
        if self.precision != "fp64":
            raise ValueError("point evaluation runs on an fp64 transform object")
        c = torch.from_numpy(np.ascontiguousarray(F.M, dtype=self._coeff_dtype())).cuda()
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        n = pts.shape[0]
        out = np.empty(n, dtype=np.complex128 if self._complex else np.float64)
        self.plan.inverse_points(c.data_ptr(), 0, pts.ctypes.data_as(_lib._dp), n, out.ctypes.data)
        return out

    # -- device-resident batch API (torch CUDA tensors)
    def make_plan(self, batch: int) -> _lib.Plan:
        return _lib.Plan(self._kind, self.l_max, batch, self.precision, self.recursion,
                         _lib.FLAG_REFINE if self.refine else 0)


class FFTSO3_complex(_Transform):
    """fdcl::FFTSO3_complex (include/fdcl_FFTSO3.hpp:27-177)."""
    _kind = _lib.SO3_COMPLEX
    _complex = True
    _so3 = True

    def _coeff_container(self, data):
        return FFTSO3_matrix_complex(self.l_max, data=data.astype(np.complex128))

    def inverse_transform(self, F, *args):
        if len(args) == 1:
            a, b, g = R_to_euler323(args[0])
        else:
            a, b, g = args
        return complex(self._points(F, np.array([[a, b, g]]))[0])

    def inverse_points(self, F, abg) -> np.ndarray:
        """Batched point evaluation at an (n, 3) array of (alpha, beta, gamma)."""
        return self._points(F, np.asarray(abg, float).reshape(-1, 3))

    def wigner_d(self, beta: float) -> FFTSO3_matrix_real:
        """d^l_mn(beta) for l <= l_max (fdcl_FFTSO3.cpp:122-125), computed on the GPU."""
        d = np.zeros(so3_ncoeff(self.l_max))
        _lib.check(_lib.lib().fftso3_wigner_d(float(beta), self.l_max, _lib.RECURSIONS[self.recursion],
                                              d.ctypes.data_as(_lib._dp)))
        return FFTSO3_matrix_real(self.l_max, data=d)

    def wigner_D(self, *args) -> FFTSO3_matrix_complex:
        """D^l_mn = d^l_mn(beta) e^{-i m alpha} e^{-i n gamma} (fdcl_FFTSO3.cpp:196-234)."""
        a, b, g = R_to_euler323(args[0]) if len(args) == 1 else args
        d = self.wigner_d(b)
        D = FFTSO3_matrix_complex(self.l_max)
        for l in range(self.l_max + 1):
            m = np.arange(-l, l + 1)
            D[l] = d[l] * np.exp(-1j * m * a)[:, None] * np.exp(-1j * m * g)[None, :]
        return D

    def check_transform(self, rng=None) -> float:
        """fdcl_FFTSO3.cpp:598-610: ||F - forward(inverse(F))|| for random F."""
        F = FFTSO3_matrix_complex(self.l_max)
        F.setRandom(rng)
        G = self.forward_transform(self.inverse_grid(F))
        return (F - G).norm()


class FFTSO3_real(FFTSO3_complex):
    """fdcl::FFTSO3_real (include/fdcl_FFTSO3.hpp:184-308)."""
    _kind = _lib.SO3_REAL
    _complex = False

    def _coeff_container(self, data):
        return FFTSO3_matrix_real(self.l_max, data=data.astype(np.float64))

    def inverse_transform(self, F, *args):
        if len(args) == 1:
            a, b, g = R_to_euler323(args[0])
        else:
            a, b, g = args
        return float(self._points(F, np.array([[a, b, g]]))[0])

    def check_transform(self, rng=None) -> float:
        """fdcl_FFTSO3.cpp:1785-1797."""
        F = FFTSO3_matrix_real(self.l_max)
        F.setRandom(rng)
        G = self.forward_transform(self.inverse_grid(F))
        return (F - G).norm()


class FFTS2_complex(_Transform):
    """fdcl::FFTS2_complex (include/fdcl_FFTS2.hpp:28-100)."""
    _kind = _lib.S2_COMPLEX
    _complex = True
    _so3 = False

    def _coeff_container(self, data):
        return FFTS2_matrix_complex(self.l_max, data=data.astype(np.complex128))

    def inverse_transform(self, F, theta: float, phi: float):
        return complex(self._points(F, np.array([[theta, phi]]))[0])

    def inverse_points(self, F, tp) -> np.ndarray:
        return self._points(F, np.asarray(tp, float).reshape(-1, 2))

    def check_transform(self, rng=None) -> float:
        """fdcl_FFTS2.cpp:302-316."""
        F = FFTS2_matrix_complex(self.l_max)
        F.setRandom(rng)
        G = self.forward_transform(self.inverse_grid(F))
        return (F - G).norm()


class FFTS2_real(FFTS2_complex):
    """fdcl::FFTS2_real (include/fdcl_FFTS2.hpp:107-160)."""
    _kind = _lib.S2_REAL
    _complex = False

    def _coeff_container(self, data):
        return FFTS2_matrix_real(self.l_max, data=data.astype(np.float64))

    def inverse_transform(self, F, theta: float, phi: float):
        return float(self._points(F, np.array([[theta, phi]]))[0])

    def check_transform(self, rng=None) -> float:
        """fdcl_FFTS2.cpp:481-493."""
        F = FFTS2_matrix_real(self.l_max)
        F.setRandom(rng)
        G = self.forward_transform(self.inverse_grid(F))
        return (F - G).norm()


def correlate_s2(F, G, *, precision: str = "fp64", recursion: str = "reference"):
    """S^2 -> SO(3) correlation of two real spherical functions (shape matching).

    F, G: FFTS2_matrix_real of one l_max.  Returns (J, (alpha, beta, gamma), R): J the
    score J(R) = sum_l G[l]^T U^l(R) F[l] on the whole (2B)^3 Euler grid (the cost of
    the reference's shape-matching example, example/example3_SSM.hpp), and the grid
    rotation that maximises it, as Euler 3-2-3 angles and as a rotation matrix.
    """
    import torch

    if F.l_max != G.l_max:
        raise ValueError("F and G must have the same l_max")
    L = F.l_max
    N = 2 * (L + 1)
    plan = _lib.Plan(_lib.SO3_REAL, L, 1, precision, recursion)
    dt = torch.float64 if precision == "fp64" else torch.float32
    f = torch.from_numpy(np.ascontiguousarray(F.M, dtype=np.float64)).to(device="cuda", dtype=dt)
    g = torch.from_numpy(np.ascontiguousarray(G.M, dtype=np.float64)).to(device="cuda", dtype=dt)
    grid = torch.empty(N ** 3, dtype=dt, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    plan.correlate_s2(f.data_ptr(), g.data_ptr(), grid.data_ptr(), s)
    (idx,), _ = plan.grid_argmax(grid.data_ptr(), s)
    k, j1, j2 = idx // (N * N), (idx // N) % N, idx % N
    abg = (float(alpha_j(L, j1)), float(beta_k(L, k)), float(alpha_j(L, j2)))
    return grid.cpu().numpy().astype(np.float64).reshape(N, N, N), abg, euler323_to_R(*abg)
