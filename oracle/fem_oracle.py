"""FP64 NumPy oracle for the FEM-elasticity / PNCG hot path of liblaf/apple.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The product (``apple_gb300``) never
imports, calls or links anything under ``oracle/``.

It restates, element by element, the arithmetic of the reference's Warp
kernels in double precision (the reference's default, ``JAX_ENABLE_X64``):

* deformation gradient and its jvp/vjp   -- ``warp/fem/func/_deformation.py:9-31``
* invariants and their gradients          -- ``func/_identity.py:9-39``, ``func/_gradient.py:9-40``
* ``lambdas`` / ``Qs`` twist modes        -- ``func/_misc.py:31-43,56-70``
* h1..h6 diag / prod / quad               -- ``func/_hess_diag.py``, ``func/_hess_prod.py``, ``func/_hess_quad.py``
* rotation-variant SVD and polar          -- ``warp/math/_rotation.py:9-22``
* ARAP                                    -- ``warp/fem/_arap.py:17-76``
* stable Neo-Hookean                      -- ``warp/fem/_stable_neo_hookean.py:17-103``
* stable Neo-Hookean muscle (G = F A)     -- ``warp/fem/_stable_neo_hookean_muscle.py:18-114``,
  ``func/_misc.py:48-53``
* per-(tet, qp) kernels with dV weighting and clamps -- ``warp/fem/_base.py:243-383``
* region precompute (dhdX, dV)            -- ``jax/fem/region/_region.py:84-108``
* DOF map                                 -- ``forward/dof_map/_dof_map.py:30-49``
* external force                          -- ``warp/potential/_ext_force.py:17-39``
* PNCG iteration (Dai-Kou beta, Jacobi preconditioner, alpha from pHp,
  Armijo backtracking)                    -- ``benches/bench_pncg_branching_backends.py:254-456,606-679``

Parity pinning: the reference's element path is pinned by golden vectors of
its own code.  ``tests/golden/make_elem_golden.py`` runs the reference's
unmodified ``warp/fem/_base.py`` kernels, the three materials, the element
functions of ``warp/fem/func`` / ``warp/math`` and ``Region.compute_grad`` on
NumPy (a stand-in for ``warp``, ``tests/golden/warp_numpy.py``), and
``tests/test_golden_reference.py`` checks this oracle against them at 1e-12
(energy density, PK1, fun, grad, hess_diag, hess_prod -- ARAP's as written
and as intended -- hess_quad, dhdX, dV).  The end-to-end PNCG solve is pinned
by the reference's known answer, the embedded-vertex ARAP solve of
``tests/forward/test_static_simulation.py:58-93`` (u4 = (0.05,-0.025,0.0375),
atol 1e-8), and the scatter by the lumped-volume sum of
``benches/test_aggregation.py:82,129``.  The PNCG iterate sequence of the
real solver (``liblaf-peach``, not vendored) has no golden vector: it follows
the in-tree proxy and stays unpinned.

The 3x3 SVD uses LAPACK (``numpy.linalg.svd``) with the rotation-variant sign
fix (det U = det V = +1, the smallest singular value carries the sign of
det F).  The reference calls ``wp.svd3`` without a sign fix-up; its reflection
convention cannot be checked here, so parity inputs avoid inverted tets.
"""

from __future__ import annotations

import dataclasses
import enum
import math
from typing import Callable

import numpy as np

SQRT2 = math.sqrt(2.0)

# ---------------------------------------------------------------------------
# element math (func/*)
# ---------------------------------------------------------------------------


def deformation_gradient(u_cell: np.ndarray, dhdX: np.ndarray) -> np.ndarray:
    """F = I + u^T dhdX  (``func/_deformation.py:15-19``).  Shapes (...,4,3)->(...,3,3)."""
    return np.einsum("...ai,...aj->...ij", u_cell, dhdX) + np.eye(3)


def deformation_gradient_jvp(dhdX: np.ndarray, p: np.ndarray) -> np.ndarray:
    """dF = p^T dhdX  (``func/_deformation.py:22-25``)."""
    return np.einsum("...ai,...aj->...ij", p, dhdX)


def deformation_gradient_vjp(dhdX: np.ndarray, P: np.ndarray) -> np.ndarray:
    """dhdX P^T, shape (...,4,3)  (``func/_deformation.py:28-31``)."""
    return np.einsum("...aj,...ij->...ai", dhdX, P)


def I2(F: np.ndarray) -> np.ndarray:
    """||F||_F^2  (``func/_identity.py:20-28``)."""
    return np.einsum("...ij,...ij->...", F, F)


def I3(F: np.ndarray) -> np.ndarray:
    """det F  (``func/_identity.py:31-39``)."""
    return np.linalg.det(F)


def g3(F: np.ndarray) -> np.ndarray:
    """dJ/dF = [f1 x f2, f2 x f0, f0 x f1] as columns  (``func/_gradient.py:31-40``)."""
    f0, f1, f2 = F[..., :, 0], F[..., :, 1], F[..., :, 2]
    return np.stack([np.cross(f1, f2), np.cross(f2, f0), np.cross(f0, f1)], axis=-1)


def svd_rv(F: np.ndarray):
    """Rotation-variant SVD F = U diag(sigma) V^T with det U = det V = +1.

    Follows the role of ``warp/math/_rotation.py:9-13`` (``wp.svd3``)."""
    U, s, Vt = np.linalg.svd(F)
    V = np.swapaxes(Vt, -1, -2).copy()
    U = U.copy()
    s = s.copy()
    neg_u = np.linalg.det(U) < 0
    U[neg_u, :, 2] *= -1.0
    s[neg_u, 2] *= -1.0
    neg_v = np.linalg.det(V) < 0
    V[neg_v, :, 2] *= -1.0
    s[neg_v, 2] *= -1.0
    return U, s, V


def polar_rv(F: np.ndarray):
    """R = U V^T, S = V diag(sigma) V^T  (``warp/math/_rotation.py:16-22``)."""
    U, s, V = svd_rv(F)
    R = U @ np.swapaxes(V, -1, -2)
    S = np.einsum("...ik,...k,...jk->...ij", V, s, V)
    return R, S


def lambdas(sigma: np.ndarray, clamp: bool = True) -> np.ndarray:
    """2 / max(sigma_i + sigma_j, 2) for pairs (0,1),(1,2),(2,0)  (``func/_misc.py:31-43``)."""
    s0, s1, s2 = sigma[..., 0], sigma[..., 1], sigma[..., 2]
    pairs = np.stack([s0 + s1, s1 + s2, s2 + s0], axis=-1)
    if clamp:
        return 2.0 / np.maximum(pairs, 2.0)
    return 2.0 / pairs


def Qs(U: np.ndarray, V: np.ndarray):
    """Twist modes  (``func/_misc.py:56-70``)."""
    u0, u1, u2 = U[..., :, 0], U[..., :, 1], U[..., :, 2]
    v0, v1, v2 = V[..., :, 0], V[..., :, 1], V[..., :, 2]
    outer = lambda a, b: np.einsum("...i,...j->...ij", a, b)  # noqa: E731
    Q0 = (outer(u1, v0) - outer(u0, v1)) / SQRT2
    Q1 = (outer(u1, v2) - outer(u2, v1)) / SQRT2
    Q2 = (outer(u0, v2) - outer(u2, v0)) / SQRT2
    return Q0, Q1, Q2


def ddot(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    return np.einsum("...ij,...ij->...", A, B)


# h-terms -------------------------------------------------------------------


def h3_diag(dhdX, g3_):
    return deformation_gradient_vjp(dhdX, g3_) ** 2  # _hess_diag.py:29-33


def h4_diag(dhdX, U, sigma, V, clamp_lambda=True):
    lam = lambdas(sigma, clamp_lambda)  # _hess_diag.py:36-50
    out = 0.0
    for i, Q in enumerate(Qs(U, V)):
        W = deformation_gradient_vjp(dhdX, Q)
        out = out + lam[..., i, None, None] * W**2
    return out


def h5_diag(dhdX):
    t = np.einsum("...aj,...aj->...a", dhdX, dhdX)  # _hess_diag.py:53-66
    return 2.0 * np.repeat(t[..., None], 3, axis=-1)


def h3_prod(p, dhdX, g3_):
    w = deformation_gradient_vjp(dhdX, g3_)  # _hess_prod.py:29-33
    return np.einsum("...ai,...ai->...", w, p)[..., None, None] * w


def h4_prod(p, dhdX, U, sigma, V, clamp_lambda=True):
    lam = lambdas(sigma, clamp_lambda)  # _hess_prod.py:36-50
    out = 0.0
    for i, Q in enumerate(Qs(U, V)):
        w = deformation_gradient_vjp(dhdX, Q)
        out = out + (lam[..., i] * np.einsum("...ai,...ai->...", w, p))[..., None, None] * w
    return out


def h5_prod(p, dhdX):
    dF = deformation_gradient_jvp(dhdX, p)  # _hess_prod.py:53-57
    return 2.0 * deformation_gradient_vjp(dhdX, dF)


def _h6_mat(F, dF):
    f0, f1, f2 = F[..., :, 0], F[..., :, 1], F[..., :, 2]
    p0, p1, p2 = dF[..., :, 0], dF[..., :, 1], dF[..., :, 2]
    c0 = np.cross(f1, p2) - np.cross(f2, p1)
    c1 = np.cross(f2, p0) - np.cross(f0, p2)
    c2 = np.cross(f0, p1) - np.cross(f1, p0)
    return np.stack([c0, c1, c2], axis=-1)


def h6_prod(p, dhdX, F):
    dF = deformation_gradient_jvp(dhdX, p)  # _hess_prod.py:60-77
    return deformation_gradient_vjp(dhdX, _h6_mat(F, dF))


def h3_quad(p, dhdX, g3_):
    return ddot(deformation_gradient_jvp(dhdX, p), g3_) ** 2  # _hess_quad.py:30-34


def h4_quad(p, dhdX, U, sigma, V, clamp_lambda=True):
    dF = deformation_gradient_jvp(dhdX, p)  # _hess_quad.py:37-49
    lam = lambdas(sigma, clamp_lambda)
    out = 0.0
    for i, Q in enumerate(Qs(U, V)):
        out = out + lam[..., i] * ddot(Q, dF) ** 2
    return out


def h5_quad(p, dhdX):
    dF = deformation_gradient_jvp(dhdX, p)  # _hess_quad.py:52-56
    return 2.0 * ddot(dF, dF)


def h6_quad(p, dhdX, F):
    dF = deformation_gradient_jvp(dhdX, p)  # _hess_quad.py:59-74
    return ddot(dF, _h6_mat(F, dF))


# ---------------------------------------------------------------------------
# materials
# ---------------------------------------------------------------------------


class Material(enum.IntEnum):
    ARAP = 0
    STABLE_NEO_HOOKEAN = 1
    STABLE_NEO_HOOKEAN_MUSCLE = 2


def arap_energy_density(F, mu):
    R, _ = polar_rv(F)  # _arap.py:17-21
    D = F - R
    return 0.5 * mu * ddot(D, D)


def arap_pk1(F, mu):
    R, _ = polar_rv(F)  # _arap.py:24-28
    return mu[..., None, None] * (F - R)


def arap_hess_diag(F, dhdX, mu):
    U, s, V = svd_rv(F)  # _arap.py:31-40
    h = -2.0 * h4_diag(dhdX, U, s, V) + h5_diag(dhdX)
    return 0.5 * mu[..., None, None] * h


def arap_hess_prod(F, p, dhdX, mu):
    """Intended ARAP Hessian-vector product.

    ``_arap.py:43-58`` passes ``(dhdX, p)`` to ``h4_prod``/``h5_prod`` whose
    signatures are ``(p, dhdX, ...)`` (``_hess_prod.py:36-57``), swapping the
    two operands.  This restates the intended formula with the operands in
    their declared roles; ``arap_hess_prod_as_called`` reproduces the call as
    written for documentation."""
    U, s, V = svd_rv(F)
    h = -2.0 * h4_prod(p, dhdX, U, s, V) + h5_prod(p, dhdX)
    return 0.5 * mu[..., None, None] * h


def arap_hess_prod_as_called(F, p, dhdX, mu):
    """``_arap.py:55-56`` exactly as written (operands swapped)."""
    U, s, V = svd_rv(F)
    h = -2.0 * h4_prod(dhdX, p, U, s, V) + h5_prod(dhdX, p)
    return 0.5 * mu[..., None, None] * h


def arap_hess_quad(F, p, dhdX, mu):
    U, s, V = svd_rv(F)  # _arap.py:61-76
    h = -2.0 * h4_quad(p, dhdX, U, s, V) + h5_quad(p, dhdX)
    return 0.5 * mu * h


def snh_energy_density(F, mu, lam):
    """0.5 mu (I2-3) - mu (J-1) + 0.5 lambda (J-1)^2  (``_stable_neo_hookean.py:17-27``)."""
    J = I3(F)
    return 0.5 * mu * (I2(F) - 3.0) - mu * (J - 1.0) + 0.5 * lam * (J - 1.0) ** 2


def snh_pk1(F, mu, lam):
    J = I3(F)  # _stable_neo_hookean.py:30-39
    d2 = 0.5 * mu
    d3 = -mu + lam * (J - 1.0)
    return d2[..., None, None] * (2.0 * F) + d3[..., None, None] * g3(F)


def snh_hess_diag(F, dhdX, mu, lam):
    J = I3(F)  # _stable_neo_hookean.py:42-67 (h6 diag is identically 0)
    G3 = g3(F)
    return lam[..., None, None] * h3_diag(dhdX, G3) + (0.5 * mu)[..., None, None] * h5_diag(dhdX)


def snh_hess_prod(F, p, dhdX, mu, lam):
    J = I3(F)  # _stable_neo_hookean.py:70-84
    G3 = g3(F)
    d2 = 0.5 * mu
    d3 = -mu + lam * (J - 1.0)
    return (
        lam[..., None, None] * h3_prod(p, dhdX, G3)
        + d2[..., None, None] * h5_prod(p, dhdX)
        + d3[..., None, None] * h6_prod(p, dhdX, F)
    )


def snh_hess_quad(F, p, dhdX, mu, lam):
    J = I3(F)  # _stable_neo_hookean.py:87-103
    G3 = g3(F)
    d2 = 0.5 * mu
    d3 = -mu + lam * (J - 1.0)
    return lam * h3_quad(p, dhdX, G3) + d2 * h5_quad(p, dhdX) + d3 * h6_quad(p, dhdX, F)


def activation_mat33(a):
    """A = I + [[a0, a3, a4], [a3, a1, a5], [a4, a5, a2]]  (``func/_misc.py:48-53``)."""
    a = np.asarray(a, np.float64)
    A = np.empty(a.shape[:-1] + (3, 3))
    A[..., 0, 0], A[..., 1, 1], A[..., 2, 2] = 1.0 + a[..., 0], 1.0 + a[..., 1], 1.0 + a[..., 2]
    A[..., 0, 1] = A[..., 1, 0] = a[..., 3]
    A[..., 0, 2] = A[..., 2, 0] = a[..., 4]
    A[..., 1, 2] = A[..., 2, 1] = a[..., 5]
    return A


def snh_pk1_dir(F, X, mu, lam):
    """Directional derivative of ``snh_pk1`` at F along X: mu X + lambda (g3:X) g3 + d3 dg3[X]."""
    G3 = g3(F)
    d3 = -mu + lam * (I3(F) - 1.0)
    return (mu[..., None, None] * X + (lam * ddot(G3, X))[..., None, None] * G3
            + d3[..., None, None] * _h6_mat(F, X))


def muscle_activation_vjp(F, W0, A, mu, lam):
    """d/da [P(F A) A^T : W0] for one cell (mu, lambda already times dV), with
    W0 = sum_a w_a dhdX_a^T.  With G = F A, W' = W0 A, P = snh_pk1(G):
    d/dA = A^-1 (G^T dP[W'] + W'^T P) (A symmetric), and
    d/da = (Z00, Z11, Z22, Z01 + Z10, Z02 + Z20, Z12 + Z21)."""
    G = F @ A
    Wp = W0 @ A
    P = snh_pk1(G, mu, lam)
    dP = snh_pk1_dir(G, Wp, mu, lam)
    T = np.swapaxes(G, -1, -2) @ dP + np.swapaxes(Wp, -1, -2) @ P
    Z = np.linalg.solve(A, T)
    return np.stack([Z[..., 0, 0], Z[..., 1, 1], Z[..., 2, 2], Z[..., 0, 1] + Z[..., 1, 0],
                     Z[..., 0, 2] + Z[..., 2, 0], Z[..., 1, 2] + Z[..., 2, 1]], axis=-1)


# ---------------------------------------------------------------------------
# region precompute (jax/fem/region/_region.py:84-108, element/_tetra.py:37-45)
# ---------------------------------------------------------------------------

DHDR = np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
QUAD_WEIGHT = 1.0 / 6.0  # quadrature/_tetra.py:14-15


def region_compute_grad(points: np.ndarray, cells: np.ndarray, fraction: np.ndarray | None = None):
    """Returns (dhdX (N_t,4,3), dV (N_t,)) with dV = det(Dm) / 6 * fraction."""
    X = points[cells].astype(np.float64)  # (c, a, I)
    dXdr = np.einsum("caI,aJ->cIJ", X, DHDR)
    drdX = np.linalg.inv(dXdr)
    dV = np.linalg.det(dXdr) * QUAD_WEIGHT
    dhdX = np.einsum("aI,cIJ->caJ", DHDR, drdX)
    if fraction is not None:
        dV = dV * fraction  # warp/fem/_base.py:104
    return dhdX, dV


# ---------------------------------------------------------------------------
# per-(tet, qp) kernels (warp/fem/_base.py:243-383)
# ---------------------------------------------------------------------------


@dataclasses.dataclass
class FemPotential:
    material: Material
    cells: np.ndarray  # (N_t, 4) int
    dhdX: np.ndarray  # (N_t, 4, 3)
    dV: np.ndarray  # (N_t,)
    mu: np.ndarray  # (N_t,)
    lam: np.ndarray | None = None  # (N_t,)
    clamp_hess_diag: bool = True
    clamp_hess_quad: bool = True
    activation: np.ndarray | None = None  # (N_t, 6), muscle only

    @classmethod
    def from_mesh(cls, material, points, cells, mu, lam=None, fraction=None, activation=None):
        dhdX, dV = region_compute_grad(points, cells, fraction)
        mu = np.broadcast_to(np.asarray(mu, np.float64), (cells.shape[0],)).copy()
        if lam is not None:
            lam = np.broadcast_to(np.asarray(lam, np.float64), (cells.shape[0],)).copy()
        if activation is not None:
            activation = np.broadcast_to(np.asarray(activation, np.float64), (cells.shape[0], 6)).copy()
        return cls(Material(material), np.asarray(cells), dhdX, dV, mu, lam, activation=activation)

    @property
    def muscle(self) -> bool:
        return self.material == Material.STABLE_NEO_HOOKEAN_MUSCLE

    def _A(self):
        a = self.activation if self.activation is not None else np.zeros((self.cells.shape[0], 6))
        return activation_mat33(a)

    def _F(self, u):
        return deformation_gradient(u[self.cells], self.dhdX)

    def _G_dhdX(self, u):
        """(F, dhdX) of the energy: the muscle evaluates at G = F A with dhdX A
        (``_stable_neo_hookean_muscle.py:18-114``)."""
        F = self._F(u)
        if not self.muscle:
            return F, self.dhdX
        A = self._A()
        return F @ A, self.dhdX @ A

    def energy_density(self, u):
        if self.material == Material.ARAP:
            return arap_energy_density(self._F(u), self.mu)
        G, _ = self._G_dhdX(u)
        return snh_energy_density(G, self.mu, self.lam)

    def pk1(self, u):
        if self.material == Material.ARAP:
            return arap_pk1(self._F(u), self.mu)
        G, _ = self._G_dhdX(u)
        P = snh_pk1(G, self.mu, self.lam)
        if self.muscle:
            P = P @ np.swapaxes(self._A(), -1, -2)  # (dPsi/dI2 g2 + dPsi/dI3 g3) A^T
        return P

    def fun(self, u) -> float:
        """Sum_e Psi_e dV_e  (``_base.py:243-263``)."""
        return float(np.sum(self.energy_density(u) * self.dV))

    def _scatter(self, n_points, per_elem):
        out = np.zeros((n_points, 3))
        np.add.at(out, self.cells.reshape(-1), per_elem.reshape(-1, 3))
        return out

    def grad(self, u) -> np.ndarray:
        """g_a += dV P dhdX_a^T  (``_base.py:265-291``)."""
        g = deformation_gradient_vjp(self.dhdX, self.pk1(u)) * self.dV[:, None, None]
        return self._scatter(u.shape[0], g)

    def hess_diag(self, u) -> np.ndarray:
        """max(dV h_diag, 0) scattered  (``_base.py:293-324``)."""
        F, dhdX = self._G_dhdX(u)
        if self.material == Material.ARAP:
            h = arap_hess_diag(F, dhdX, self.mu)
        else:
            h = snh_hess_diag(F, dhdX, self.mu, self.lam)
        h = h * self.dV[:, None, None]
        if self.clamp_hess_diag:
            h = np.maximum(h, 0.0)
        return self._scatter(u.shape[0], h)

    def hess_prod(self, u, p) -> np.ndarray:
        """dV H_e p_e scattered  (``_base.py:326-351``)."""
        F, dhdX = self._G_dhdX(u)
        pc = p[self.cells]
        if self.material == Material.ARAP:
            h = arap_hess_prod(F, pc, dhdX, self.mu)
        else:
            h = snh_hess_prod(F, pc, dhdX, self.mu, self.lam)
        return self._scatter(u.shape[0], h * self.dV[:, None, None])

    def hess_quad_elems(self, u, p) -> np.ndarray:
        F, dhdX = self._G_dhdX(u)
        pc = p[self.cells]
        if self.material == Material.ARAP:
            h = arap_hess_quad(F, pc, dhdX, self.mu)
        else:
            h = snh_hess_quad(F, pc, dhdX, self.mu, self.lam)
        h = h * self.dV
        if self.clamp_hess_quad:
            h = np.maximum(h, 0.0)
        return h

    def hess_quad(self, u, p) -> float:
        """Sum_e max(dV p^T H_e p, 0)  (``_base.py:353-383``)."""
        return float(np.sum(self.hess_quad_elems(u, p)))

    def grad_param_vjp(self, u, w):
        """d(w . grad(u))/d mu_c and d/d lambda_c per cell: the backward of the
        grad kernel on the material arrays (``_base.py:80-117`` with Warp's tape;
        ``utils/_material.py:34-38``).  grad is linear in mu and lambda:
        SNH P = mu (F - cof F) + lambda (J-1) cof F  (``_stable_neo_hookean.py:30-39``),
        ARAP P = mu (F - R)  (``_arap.py:24-28``)."""
        F, dhdX = self._G_dhdX(u)
        W = deformation_gradient_jvp(dhdX, w[self.cells])  # sum_a w_a (x) dhdX_a (muscle: dhdX_a A)
        if self.material == Material.ARAP:
            R, _ = polar_rv(F)
            return ddot(F - R, W) * self.dV, None
        C = g3(F)
        J = I3(F)
        dmu = ddot(F - C, W) * self.dV
        dlam = (J - 1.0) * ddot(C, W) * self.dV
        return dmu, dlam

    def grad_activation_vjp(self, u, w):
        """d(w . grad(u))/d activation per cell, (N_t, 6): the backward of the
        muscle grad kernel on ``activation`` (``_stable_neo_hookean_muscle.py:30-39``)."""
        if not self.muscle:
            raise ValueError("not a muscle potential")
        F = self._F(u)
        W0 = deformation_gradient_jvp(self.dhdX, w[self.cells])
        return muscle_activation_vjp(F, W0, self._A(), self.mu * self.dV, self.lam * self.dV)


@dataclasses.dataclass
class ExternalForce:
    """W = -sum f.u, grad = -f  (``warp/potential/_ext_force.py:17-39,80-90``)."""

    indices: np.ndarray
    force: np.ndarray  # (n, 3)

    def fun(self, u) -> float:
        return float(-np.sum(self.force * u[self.indices]))

    def grad(self, u) -> np.ndarray:
        out = np.zeros_like(u, dtype=np.float64)
        np.add.at(out, self.indices, -self.force)
        return out


@dataclasses.dataclass
class DofMap:
    """``forward/dof_map/_dof_map.py:10-49``; mask per component (``_builder.py:101-113``)."""

    n_points: int
    fixed_mask: np.ndarray  # (N_v, 3) bool
    fixed_values: np.ndarray  # (N_v, 3)

    @property
    def free_indices(self):
        return np.flatnonzero(~self.fixed_mask.reshape(-1))

    @property
    def fixed_indices(self):
        return np.flatnonzero(self.fixed_mask.reshape(-1))

    def to_free(self, full):
        return full.reshape(-1)[self.free_indices]

    def to_full(self, free):
        r = np.empty(self.n_points * 3)
        r[self.fixed_indices] = self.fixed_values.reshape(-1)[self.fixed_indices]
        r[self.free_indices] = free
        return r.reshape(self.n_points, 3)

    def to_full_grad(self, free):
        r = np.empty(self.n_points * 3)
        r[self.fixed_indices] = 0.0
        r[self.free_indices] = free
        return r.reshape(self.n_points, 3)


@dataclasses.dataclass
class Model:
    """Sum of potentials with zero-then-accumulate (``warp/model/_model.py:13-36``)
    behind the free-DOF problem of ``forward/_problem.py:24-59``."""

    dof_map: DofMap
    potentials: list
    ext_force: ExternalForce | None = None

    def fun(self, u):
        f = sum(p.fun(u) for p in self.potentials)
        if self.ext_force is not None:
            f += self.ext_force.fun(u)
        return f

    def grad(self, u):
        g = np.zeros((u.shape[0], 3))
        for p in self.potentials:
            g += p.grad(u)
        if self.ext_force is not None:
            g += self.ext_force.grad(u)
        return g

    def hess_diag(self, u):
        d = np.zeros((u.shape[0], 3))
        for p in self.potentials:
            d += p.hess_diag(u)
        return d

    def hess_prod(self, u, v):
        d = np.zeros((u.shape[0], 3))
        for p in self.potentials:
            d += p.hess_prod(u, v)
        return d

    def hess_quad(self, u, v):
        return sum(p.hess_quad(u, v) for p in self.potentials)


# ---------------------------------------------------------------------------
# PNCG (benches/bench_pncg_branching_backends.py:254-456,606-679)
# ---------------------------------------------------------------------------


class Result(enum.IntEnum):
    PRIMARY_SUCCESS = 0
    MAX_STEPS_REACHED = 1
    LINE_SEARCH_FAILED = 2
    NAN_ENCOUNTERED = 3


@dataclasses.dataclass
class PncgStats:
    result: Result
    n_steps: int
    grad_norm: float
    grad_norm_first: float
    energy: float
    alpha: list
    beta: list
    line_search_steps: list
    energies: list


def preconditioner(hess_diag_free: np.ndarray) -> np.ndarray:
    """1/|d| with zeros replaced by the mean of the positive entries (proxy :407-410)."""
    d = np.abs(hess_diag_free)
    pos = d > 0.0
    mean = d[pos].mean() if np.any(pos) else 1.0
    d = np.where(pos, d, mean)
    return 1.0 / d


def dai_kou_beta(grad, prev_grad, prev_direction, precond) -> float:
    """Proxy :663-679."""
    y = grad - prev_grad
    ydp = float(np.dot(y, prev_direction))
    safe = ydp if abs(ydp) > 1.0e-12 else 1.0
    Py = precond * y
    beta = np.dot(grad, Py) / safe - (np.dot(y, Py) / safe) * (np.dot(prev_direction, grad) / safe)
    return float(beta) if abs(ydp) > 1.0e-12 else math.inf


def initial_alpha(gd: float, hq: float, overstep: float = 1.0) -> float:
    """Proxy :606-610 (the proxy passes overstep=4; see ``pncg_minimize``)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        alpha = np.float64(-gd) / np.float64(hq)
    alpha = float(np.nan_to_num(alpha, nan=0.0, neginf=0.0, posinf=1.0))
    if not (alpha > 0.0 and math.isfinite(alpha)):
        alpha = 1.0
    return alpha * overstep


def pncg_minimize(
    fun: Callable,
    grad: Callable,
    hess_diag: Callable,
    hess_quad: Callable,
    x0: np.ndarray,
    *,
    max_steps: int = 1500,
    rtol: float = 1e-9,
    atol: float = 0.0,
    max_backtracking_steps: int = 8,
    armijo_c: float = 1.0e-4,
    overstep: float = 1.0,
    beta_max: float = 10.0,
    record: bool = False,
):
    """PNCG on free-space vectors, following the proxy loop step by step.

    Termination (not in the proxy, which runs a fixed count): converged when
    ||g|| <= max(atol, rtol ||g_0||) at the top of an iteration; a failed line
    search along the steepest-descent direction ends with LINE_SEARCH_FAILED.

    ``overstep`` multiplies the first trial step alpha_0 = -g.p / p.Hp.  The
    proxy uses 4 (:606-610); with 4, the reference's only end-to-end test
    (``tests/forward/test_static_simulation.py:58-93``) stalls near 6e-6 error
    because the first accepted trial is 2 alpha_0, a zero-decrease step on a
    quadratic.  The default 1 (the plain PNCG step) reaches that test's
    answer to 1e-9.
    """
    x = np.array(x0, dtype=np.float64)
    value = fun(x)
    g0 = grad(x)
    gnorm0 = float(np.linalg.norm(g0))
    prev_grad = g0
    prev_dir = np.zeros_like(x)
    stats = PncgStats(Result.MAX_STEPS_REACHED, 0, gnorm0, gnorm0, value, [], [], [], [])
    for i in range(max_steps):
        value = fun(x)
        g = grad(x)
        P = preconditioner(hess_diag(x))
        gnorm = float(np.linalg.norm(g))
        stats.grad_norm = gnorm
        stats.energy = value
        if not (math.isfinite(gnorm) and math.isfinite(value)):
            stats.result = Result.NAN_ENCOUNTERED
            return x, stats
        if gnorm <= max(atol, rtol * gnorm0):
            stats.result = Result.PRIMARY_SUCCESS
            return x, stats
        beta = dai_kou_beta(g, prev_grad, prev_dir, P)
        if i == 0 or not (math.isfinite(beta) and abs(beta) <= beta_max):
            beta = 0.0
        steep = -P * g
        d = steep + beta * prev_dir
        gd = float(np.dot(g, d))
        if not (math.isfinite(gd) and gd < 0.0):
            beta = 0.0
            d = steep
            gd = float(np.dot(g, d))
        hq = hess_quad(x, d)
        alpha = initial_alpha(gd, hq, overstep)
        trial = x + alpha * d
        tv = fun(trial)
        accepted = math.isfinite(tv) and tv <= value + armijo_c * alpha * gd
        ls = 0
        while (not accepted) and ls < max_backtracking_steps and alpha > 0.0:
            alpha *= 0.5
            trial = x + alpha * d
            tv = fun(trial)
            accepted = math.isfinite(tv) and tv <= value + armijo_c * alpha * gd
            ls += 1
        if record:
            stats.alpha.append(alpha if accepted else 0.0)
            stats.beta.append(beta)
            stats.line_search_steps.append(ls)
            stats.energies.append(tv if accepted else value)
        stats.n_steps = i + 1
        if accepted:
            x = trial
            value = tv
        elif beta == 0.0:
            stats.result = Result.LINE_SEARCH_FAILED
            return x, stats
        prev_grad = g
        prev_dir = d
    stats.energy = fun(x)
    stats.grad_norm = float(np.linalg.norm(grad(x)))
    if stats.grad_norm <= max(atol, rtol * gnorm0):
        stats.result = Result.PRIMARY_SUCCESS
    return x, stats


def solve_model(model: Model, u0_full: np.ndarray | None = None, **kw):
    """``Forward.step()`` equivalent: PNCG over the free DOFs (``forward/_forward.py:52-56``)."""
    dm = model.dof_map
    if u0_full is None:
        x0 = np.zeros(dm.free_indices.size)
    else:
        x0 = dm.to_free(np.asarray(u0_full, np.float64))
    fun = lambda x: model.fun(dm.to_full(x))  # noqa: E731
    grad = lambda x: dm.to_free(model.grad(dm.to_full(x)))  # noqa: E731
    hd = lambda x: dm.to_free(model.hess_diag(dm.to_full(x)))  # noqa: E731
    hq = lambda x, p: model.hess_quad(dm.to_full(x), dm.to_full_grad(p))  # noqa: E731
    x, stats = pncg_minimize(fun, grad, hd, hq, x0, **kw)
    return dm.to_full(x), stats


def dense_hessian_free(model: Model, u: np.ndarray) -> np.ndarray:
    """H(u) on the free DOFs, column by column from hess_prod (small meshes)."""
    dm = model.dof_map
    free = dm.free_indices
    H = np.empty((free.size, free.size))
    for j, k in enumerate(free):
        e = np.zeros(u.size)
        e[k] = 1.0
        H[:, j] = model.hess_prod(u, e.reshape(-1, 3)).reshape(-1)[free]
    return 0.5 * (H + H.T)


def adjoint_dense(model: Model, u: np.ndarray, rhs: np.ndarray) -> np.ndarray:
    """lam with H(u) lam = rhs on the free DOFs (0 on fixed), by a dense solve."""
    dm = model.dof_map
    lam_free = np.linalg.solve(dense_hessian_free(model, u), rhs.reshape(-1)[dm.free_indices])
    return dm.to_full_grad(lam_free)


def equilibrium_param_grad(model: Model, potential: FemPotential, u: np.ndarray, dLdu: np.ndarray):
    """Implicit differentiation of g(u*, theta) = 0 (the reference's inverse
    recipe, ``exp/2025/09/24/inverse-grin/src/32-inverse.py:223-300``):
    dL/dmu, dL/dlambda = -d(lam . g)/d(mu, lambda), H lam = dL/du."""
    lam = adjoint_dense(model, u, dLdu)
    dmu, dlam = potential.grad_param_vjp(u, lam)
    return -dmu, (None if dlam is None else -dlam), lam


def equilibrium_activation_grad(model: Model, potential: FemPotential, u: np.ndarray, dLdu: np.ndarray):
    """dL/d activation = -d(lam . g)/d activation with H lam = dL/du (muscle)."""
    lam = adjoint_dense(model, u, dLdu)
    return -potential.grad_activation_vjp(u, lam), lam


# ---------------------------------------------------------------------------
# known-answer helpers
# ---------------------------------------------------------------------------


def lumped_volume(points: np.ndarray, cells: np.ndarray) -> np.ndarray:
    """|det|/6 /4 to each corner  (``benches/test_aggregation.py:30-54``)."""
    p = points[cells]
    D = np.stack([p[:, 0] - p[:, 3], p[:, 1] - p[:, 3], p[:, 2] - p[:, 3]], axis=-1)
    vol = np.abs(np.linalg.det(D)) / 6.0
    out = np.zeros(points.shape[0])
    np.add.at(out, cells.reshape(-1), np.repeat(vol / 4.0, 4))
    return out


def lame_converter(E, nu):
    """(lambda, mu) from (E, nu)  (``common/_moduli.py:5-10``)."""
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    return lam, mu
