"""CPU checks of the muscle oracle: every derivative against central
differences of the one below it, and the zero-activation case against the
stable Neo-Hookean."""

import numpy as np

from apple_gb300 import meshgen
from oracle import fem_oracle as O


def _pot(seed=0, act_scale=0.1):
    rng = np.random.default_rng(seed)
    m = meshgen.grid(2, 2, 3)
    nt = m.n_cells
    act = act_scale * rng.normal(size=(nt, 6))
    pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN_MUSCLE, m.points, m.cells,
                                   mu=rng.uniform(1, 2, nt), lam=rng.uniform(3, 5, nt), activation=act)
    u = 0.05 * rng.normal(size=(m.n_points, 3))
    return m, pot, u, rng


def _fd(f, x, h=1e-6):
    out = np.zeros_like(x)
    for i in np.ndindex(x.shape):
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        out[i] = (f(xp) - f(xm)) / (2 * h)
    return out


def test_muscle_grad_hess_match_differences():
    m, pot, u, rng = _pot()
    p = rng.normal(size=u.shape)
    g = pot.grad(u)
    assert np.abs(g - _fd(pot.fun, u)).max() < 1e-7 * np.abs(g).max()
    hp = pot.hess_prod(u, p)
    fd = (pot.grad(u + 1e-6 * p) - pot.grad(u - 1e-6 * p)) / 2e-6
    assert np.abs(hp - fd).max() < 1e-7 * np.abs(hp).max()
    assert abs(pot.hess_quad(u, p) - np.sum(p * hp)) < 1e-9 * abs(np.sum(p * hp))
    hd = pot.hess_diag(u)
    ex = np.zeros_like(u)
    for i in np.ndindex(u.shape):
        e = np.zeros_like(u)
        e[i] = 1.0
        ex[i] = max(np.sum(e * pot.hess_prod(u, e)), 0.0)
    # per-element clamps at max(., 0) only differ from the exact diagonal on non-convex elements
    assert np.abs(hd - ex).max() < 1e-9 * np.abs(ex).max()


def test_muscle_material_and_activation_vjp_match_differences():
    m, pot, u, rng = _pot(seed=1)
    w = rng.normal(size=u.shape)
    act0, mu0 = pot.activation.copy(), pot.mu.copy()

    def wg_act(a):
        pot.activation = a
        return float(np.sum(w * pot.grad(u)))

    def wg_mu(mu):
        pot.mu = mu
        return float(np.sum(w * pot.grad(u)))

    da = pot.grad_activation_vjp(u, w)
    fda = _fd(wg_act, act0)
    pot.activation = act0
    assert np.abs(da - fda).max() < 1e-7 * np.abs(da).max()
    dmu, _ = pot.grad_param_vjp(u, w)
    fdm = _fd(wg_mu, mu0)
    pot.mu = mu0
    assert np.abs(dmu - fdm).max() < 1e-7 * np.abs(dmu).max()


def test_zero_activation_is_stable_neo_hookean():
    m, pot, u, rng = _pot(seed=2, act_scale=0.0)
    snh = O.FemPotential(O.Material.STABLE_NEO_HOOKEAN, pot.cells, pot.dhdX, pot.dV, pot.mu, pot.lam)
    p = rng.normal(size=u.shape)
    assert pot.fun(u) == snh.fun(u)
    np.testing.assert_array_equal(pot.grad(u), snh.grad(u))
    np.testing.assert_allclose(pot.hess_prod(u, p), snh.hess_prod(u, p), rtol=1e-14, atol=1e-14)


def test_activation_matrix_layout():
    a = np.arange(1.0, 7.0)
    A = O.activation_mat33(a)
    np.testing.assert_array_equal(A, [[2.0, 4.0, 5.0], [4.0, 3.0, 6.0], [5.0, 6.0, 4.0]])
