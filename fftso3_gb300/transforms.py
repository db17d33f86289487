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
from .rotation import R_to_euler323, euler323_to_R, expm_SO3


def beta_k(l_max: int, k) -> np.ndarray:
    """beta_k = (2k+1) pi / (4B) (fdcl_FFTSO3.cpp:578-581)."""
    B = l_max + 1
    return (2.0 * np.asarray(k, float) + 1.0) * np.pi / 4.0 / B


def alpha_j(l_max: int, j) -> np.ndarray:
    """alpha_j = gamma_j = j pi / B (fdcl_FFTSO3.cpp:583-591)."""
    return np.asarray(j, float) * np.pi / (l_max + 1)


def _rsph(l: int) -> np.ndarray:
    """matrix2rsph T(l) (fdcl_FFTSO3.cpp:1107-1139): row a, column c, indices shifted by l."""
    W = 2 * l + 1
    T = np.zeros((W, W), complex)
    s = 1.0 / np.sqrt(2.0)
    for a in range(-l, l + 1):
        sg = -1.0 if (a & 1) else 1.0
        if a < 0:
            T[a + l, a + l] = 1j * s
            T[a + l, -a + l] = -1j * s * sg
        elif a == 0:
            T[l, l] = 1.0
        else:
            T[a + l, -a + l] = s
            T[a + l, a + l] = sg * s
    return T


def real_from_wigner_D(D) -> FFTSO3_matrix_real:
    """Real harmonics U^l = Re(conj(T) D^l T^T) of a Wigner-D container (fdcl_FFTSO3.cpp:1062-1105)."""
    U = FFTSO3_matrix_real(D.l_max)
    for l in range(D.l_max + 1):
        T = _rsph(l)
        U[l] = np.real(np.conj(T) @ D[l] @ T.T)
    return U


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
                 refine: bool = False, exact_inverse: bool = False):
        self.precision = precision
        self.recursion = recursion
        self.refine = refine
        self.exact_inverse = exact_inverse
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

    def _flags(self) -> int:
        return (_lib.FLAG_REFINE if self.refine else 0) | (_lib.FLAG_EXACT_INVERSE if self.exact_inverse else 0)

    @property
    def plan(self) -> _lib.Plan:
        if self._plan is None:
            self._plan = _lib.Plan(self._kind, self.l_max, 1, self.precision, self.recursion,
                                   self._flags())
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

    def derivative(self, F, axis: int):
        """Coefficients of f_i(R) = d/dt f(R exp(t e_i)) at t = 0 (i = axis in 1..3), computed on the GPU
        (fftso3_derivative): F^l (u_i^l)^T with u_i the matrices of deriv_wigner_D / deriv_real_harmonics.
        SO(3) only."""
        import torch

        if not self._so3:
            raise ValueError("derivatives are defined for SO(3) functions")
        self.init(F.l_max)
        c = torch.from_numpy(np.ascontiguousarray(F.M, dtype=self._coeff_dtype())).cuda()
        out = torch.empty_like(c)
        s = torch.cuda.current_stream().cuda_stream
        self.plan.derivative(c.data_ptr(), int(axis), out.data_ptr(), s)
        torch.cuda.synchronize()
        return self._coeff_container(out.cpu().numpy())

    # -- device-resident batch API (torch CUDA tensors)
    def make_plan(self, batch: int) -> _lib.Plan:
        return _lib.Plan(self._kind, self.l_max, batch, self.precision, self.recursion,
                         self._flags())


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

    def deriv_wigner_D(self) -> list:
        """[None, u1, u2, u3]: d/dt D(exp(t e_i)) at t = 0 for each l (fdcl_FFTSO3.cpp:417-453),
        so that d/dt D(R exp(t e_i)) = D(R) u_i."""
        u = [None] + [FFTSO3_matrix_complex(self.l_max) for _ in range(3)]
        for l in range(self.l_max + 1):
            m = np.arange(-l, l + 1)
            W = 2 * l + 1
            u3 = np.zeros((W, W), complex)
            u3[m + l, m + l] = -1j * m
            u1 = np.zeros((W, W), complex)
            u2 = np.zeros((W, W), complex)
            up = m[:-1]                      # n = m + 1
            c = np.sqrt((l + up + 1.0) * (l - up))
            u2[up + l, up + 1 + l] = 0.5 * c
            u1[up + l, up + 1 + l] = -0.5j * c
            dn = m[1:]                       # n = m - 1
            c = np.sqrt((l - dn + 1.0) * (l + dn))
            u2[dn + l, dn - 1 + l] = -0.5 * c
            u1[dn + l, dn - 1 + l] = -0.5j * c
            u[1][l], u[2][l], u[3][l] = u1, u2, u3
        return u

    def check_deriv_wigner_D(self, eps: float = 1e-6) -> float:
        """fdcl_FFTSO3.cpp:455-492: the derivatives against (D(exp(eps e_i)) - D(I)) / eps."""
        u = self.deriv_wigner_D()
        D0 = self.wigner_D(0.0, 0.0, 0.0)
        err = np.zeros(self.l_max)
        for i in range(1, 4):
            e = np.zeros(3)
            e[i - 1] = eps
            D1 = self.wigner_D(expm_SO3(e))
            for l in range(1, self.l_max + 1):
                err[l - 1] += np.linalg.norm((D1[l] - D0[l]) / eps - u[i][l]) / np.linalg.norm(u[i][l])
        return float(err.max() * 1e-9)

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

    def real_harmonics(self, *args) -> FFTSO3_matrix_real:
        """U^l = Re(conj(T) D^l T^T), T = matrix2rsph (fdcl_FFTSO3.cpp:1062-1139)."""
        return real_from_wigner_D(self.wigner_D(*args))

    def deriv_real_harmonics(self) -> list:
        """[None, u1, u2, u3]: d/dt U(exp(t e_i)) at t = 0 (fdcl_FFTSO3.cpp:1577-1645), so that
        d/dt U(R exp(t e_i)) = U(R) u_i."""
        u = [None] + [FFTSO3_matrix_real(self.l_max) for _ in range(3)]
        for l in range(self.l_max + 1):
            W = 2 * l + 1
            M = [np.zeros((W, W)) for _ in range(3)]
            ix = lambda m: m + l  # noqa: E731
            for p in range(1, l + 1):
                M[2][ix(p), ix(-p)] = -p          # u3(l, m, -m) = -m
                M[2][ix(-p), ix(p)] = p
            for p in range(2, l + 1):
                t = 0.5 * np.sqrt((l + p) * (l - p + 1.0))
                M[1][ix(p), ix(p - 1)] = t
                M[1][ix(-p), ix(-p + 1)] = t
                M[0][ix(p), ix(-p + 1)] = (p + (-p + 1)) * t
                M[0][ix(-p), ix(p - 1)] = (-p + (p - 1)) * t
                q = p - 1
                t = 0.5 * np.sqrt((l - q) * (l + q + 1.0))
                M[1][ix(q), ix(q + 1)] = -t
                M[1][ix(-q), ix(-q - 1)] = -t
                M[0][ix(q), ix(-q - 1)] = -(q + (-q - 1)) * t
                M[0][ix(-q), ix(q + 1)] = -(-q + (q + 1)) * t
            if l >= 1:
                t = np.sqrt(l * (l + 1.0) / 2.0)
                M[1][ix(1), ix(0)] = t
                M[1][ix(0), ix(1)] = -t
                M[0][ix(-1), ix(0)] = -t
                M[0][ix(0), ix(-1)] = t
            u[1][l], u[2][l], u[3][l] = M
        return u

    def check_deriv_real_harmonics(self, eps: float = 1e-6) -> float:
        """fdcl_FFTSO3.cpp:1648-1681: the derivatives against (U(exp(eps e_i)) - U(I)) / eps."""
        u = self.deriv_real_harmonics()
        U0 = self.real_harmonics(0.0, 0.0, 0.0)
        err = 0.0
        for i in range(1, 4):
            e = np.zeros(3)
            e[i - 1] = eps
            U1 = self.real_harmonics(expm_SO3(e))
            for l in range(1, self.l_max + 1):
                err += np.linalg.norm((U1[l] - U0[l]) / eps - u[i][l]) / np.linalg.norm(u[i][l])
        return float(err * 1e-9)

    def check_Clebsch_Gordon(self, l1: int = 3, l2: int = 5, rng=None) -> float:
        """fdcl_FFTSO3.cpp:1683+: ||U^{l1} (x) U^{l2} - c ((+)_l U^l) c^H|| at a random rotation."""
        from .clebsch_gordan import Clebsch_Gordon_real

        rng = np.random.default_rng(rng)
        a, b, g = rng.uniform(0, 2 * np.pi), rng.uniform(0, np.pi), rng.uniform(0, 2 * np.pi)
        U = FFTSO3_real(l1 + l2, recursion=self.recursion).real_harmonics(a, b, g)
        cg = Clebsch_Gordon_real()
        cg.compute(l1, l2)
        n = cg.c.shape[0]
        B = np.zeros((n, n))
        i = 0
        for l in range(abs(l1 - l2), l1 + l2 + 1):
            B[i:i + 2 * l + 1, i:i + 2 * l + 1] = U[l]
            i += 2 * l + 1
        return float(np.linalg.norm(np.kron(U[l1], U[l2]) - cg.c @ B @ cg.c.conj().T))

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


def correlate_s2(F, G, *, precision: str = "fp64", recursion: str = "reference", gradient: bool = False):
    """S^2 -> SO(3) correlation of two real spherical functions (shape matching).

    F, G: FFTS2_matrix_real of one l_max.  Returns (J, (alpha, beta, gamma), R): J the
    score J(R) = sum_l G[l]^T U^l(R) F[l] on the whole (2B)^3 Euler grid (the cost of
    the reference's shape-matching example, example/example3_SSM.hpp), and the grid
    rotation that maximises it, as Euler 3-2-3 angles and as a rotation matrix.
    With gradient=True also dJ (3, N, N, N): dJ_i(R) = d/dt J(R exp(t e_i)) at t = 0
    = sum_l G[l]^T U^l(R) u_i^l F[l] (the reference's gradient(R), example3_SSM.hpp),
    i.e. the same correlation with F[l] replaced by u_i^l F[l].
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
    J = grid.cpu().numpy().astype(np.float64).reshape(N, N, N)
    if not gradient:
        return J, abg, euler323_to_R(*abg)
    u = FFTSO3_real(L).deriv_real_harmonics()
    dJ = np.empty((3, N, N, N))
    for i in range(1, 4):
        Fi = np.concatenate([u[i][l] @ F[l] for l in range(L + 1)])
        fi = torch.from_numpy(Fi).to(device="cuda", dtype=dt)
        plan.correlate_s2(fi.data_ptr(), g.data_ptr(), grid.data_ptr(), s)
        dJ[i - 1] = grid.cpu().numpy().astype(np.float64).reshape(N, N, N)
    return J, abg, euler323_to_R(*abg), dJ
