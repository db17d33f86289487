"""3-2-3 Euler angles <-> rotation matrices, as used by the f(R) overloads of
the transforms (fdcl_FFTSO3.cpp:934-941, :1246-1253, :568-576, :1158-1167).

Restates misc_matrix_func.cpp:144-177 (R2Euler323, Euler3232R); vectorised
over leading axes.
"""
from __future__ import annotations

import numpy as np


def euler323_to_R(a, b, g) -> np.ndarray:
    """Euler3232R (misc_matrix_func.cpp:168-177); returns (..., 3, 3)."""
    a, b, g = np.broadcast_arrays(np.asarray(a, float), np.asarray(b, float), np.asarray(g, float))
    ca, sa, cb, sb, cg, sg = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(g), np.sin(g)
    R = np.empty(a.shape + (3, 3))
    R[..., 0, 0] = ca * cb * cg - sa * sg
    R[..., 0, 1] = -cg * sa - ca * cb * sg
    R[..., 0, 2] = ca * sb
    R[..., 1, 0] = ca * sg + cb * cg * sa
    R[..., 1, 1] = ca * cg - cb * sa * sg
    R[..., 1, 2] = sa * sb
    R[..., 2, 0] = -cg * sb
    R[..., 2, 1] = sb * sg
    R[..., 2, 2] = cb
    return R


def R_to_euler323(R) -> tuple[float, float, float]:
    """R2Euler323 (misc_matrix_func.cpp:144-166) for one 3x3 rotation."""
    R = np.asarray(R, float)
    b = float(np.arccos(np.clip(R[2, 2], -1.0, 1.0)))
    if b != 0.0:
        g = float(np.arctan2(R[2, 1], -R[2, 0]))
        a = float(np.arctan2(R[1, 2], R[0, 2]))
    else:
        a = float(np.arccos(np.clip(R[0, 0], -1.0, 1.0)) / 2.0)
        g = a
    return a, b, g


def hat(v) -> np.ndarray:
    """hat map R^3 -> so(3) (misc_matrix_func.cpp:7-17)."""
    x, y, z = (float(t) for t in v)
    return np.array([[0.0, -z, y], [z, 0.0, -x], [-y, x, 0.0]])


def expm_SO3(r) -> np.ndarray:
    """exp(hat r) by the Rodrigues formula (the rotation misc_matrix_func.cpp:49-60 computes)."""
    r = np.asarray(r, float)
    th = float(np.linalg.norm(r))
    K = hat(r)
    if th < 1e-12:
        return np.eye(3) + K
    return np.eye(3) + np.sin(th) / th * K + (1.0 - np.cos(th)) / th ** 2 * (K @ K)
