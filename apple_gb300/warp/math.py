"""``liblaf.apple.warp.math`` (warp/math/__init__.pyi, _rotation.py:9-22):
the rotation-variant SVD and polar decomposition of batches of 3x3 matrices.
These run on the host in float64 (numpy.linalg.svd with the sign fix: det U =
det V = +1, the smallest singular value carries the sign of det F) for use
outside the solver; the kernels have their own Jacobi SVD on the device."""

from __future__ import annotations

import numpy as np

__all__ = ["polar_rv", "svd_rv"]


def svd_rv(F):
    """F = U diag(sigma) V^T with det U = det V = +1 (F: (..., 3, 3))."""
    F = np.asarray(F, np.float64)
    U, s, Vt = np.linalg.svd(F)
    V = np.swapaxes(Vt, -1, -2)
    du = np.linalg.det(U) < 0
    dv = np.linalg.det(V) < 0
    U = U.copy()
    V = V.copy()
    s = s.copy()
    U[du, :, 2] *= -1.0
    s[du, 2] *= -1.0
    V[dv, :, 2] *= -1.0
    s[dv, 2] *= -1.0
    return U, s, V


def polar_rv(F):
    """F = R S with R = U V^T a rotation and S = V diag(sigma) V^T."""
    U, s, V = svd_rv(F)
    R = U @ np.swapaxes(V, -1, -2)
    S = V @ (s[..., :, None] * np.swapaxes(V, -1, -2))
    return R, S
