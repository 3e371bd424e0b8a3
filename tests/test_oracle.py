"""The FP64 oracle checked against the reference's own known answers and by
finite differences (CPU only)."""

import json
import math
import pathlib

import numpy as np
import pytest

from apple_gb300 import meshgen
from oracle import fem_oracle as O

GOLDEN = pathlib.Path(__file__).parent / "golden"


def _embedded():
    d = json.loads((GOLDEN / "embedded_tetra.json").read_text())
    pts = np.asarray(d["points"], float)
    cells = np.asarray(d["cells"], int)
    mask = np.zeros((len(pts), 3), bool)
    mask[d["fixed_vertices"]] = True
    fv = np.zeros((len(pts), 3))
    fv[d["fixed_value_vertex"]] = d["fixed_value"]
    return d, pts, cells, mask, fv


def test_embedded_vertex_known_answer():
    """tests/forward/test_static_simulation.py:58-93 of the reference."""
    d, pts, cells, mask, fv = _embedded()
    pot = O.FemPotential.from_mesh(O.Material.ARAP, pts, cells, mu=d["mu"])
    model = O.Model(O.DofMap(len(pts), mask, fv), [pot])
    u0 = model.dof_map.to_full(np.zeros(model.dof_map.free_indices.size))
    e0 = model.fun(u0)
    u, st = O.solve_model(model)
    assert st.result.name == d["result"]
    assert model.dof_map.free_indices.size == d["n_free"]
    assert math.isfinite(e0) and model.fun(u) < e0
    np.testing.assert_allclose(u[:4], fv[:4])
    np.testing.assert_allclose(u[d["expect_vertex"]], d["expect_u"], atol=d["atol"])


def test_proxy_overstep_four_does_not_reach_known_answer():
    """Documents why overstep defaults to 1: with the proxy's 4 the
    reference's end-to-end answer is not reached."""
    d, pts, cells, mask, fv = _embedded()
    pot = O.FemPotential.from_mesh(O.Material.ARAP, pts, cells, mu=1.0)
    model = O.Model(O.DofMap(len(pts), mask, fv), [pot])
    u, st = O.solve_model(model, overstep=4.0, max_steps=200)
    assert st.result.name != "PRIMARY_SUCCESS"
    assert np.abs(u[4] - d["expect_u"]).max() > 1e-7


@pytest.mark.parametrize("mesh", ["grid", "ball"])
def test_lumped_volume_sum(mesh):
    """benches/test_aggregation.py:82,129: sum of lumped volumes = mesh volume."""
    m = meshgen.grid(4, 3, 5) if mesh == "grid" else meshgen.ball(800, 200, seed=1)
    lv = O.lumped_volume(m.points, m.cells)
    assert lv.sum() == pytest.approx(m.volume(), rel=1e-12)


def _random_state(material, seed=0, n=(3, 3, 2), amp=0.15):
    rng = np.random.default_rng(seed)
    m = meshgen.grid(*n)
    nt = m.n_cells
    mu = rng.uniform(0.5, 2.0, nt)
    lam = rng.uniform(1.0, 10.0, nt) if material == O.Material.STABLE_NEO_HOOKEAN else None
    pot = O.FemPotential.from_mesh(material, m.points, m.cells, mu=mu, lam=lam)
    u = amp * rng.normal(size=(m.n_points, 3))
    p = rng.normal(size=(m.n_points, 3))
    return pot, u, p


MATERIALS = [O.Material.ARAP, O.Material.STABLE_NEO_HOOKEAN]


@pytest.mark.parametrize("material", MATERIALS)
def test_grad_matches_fd_of_fun(material):
    pot, u, p = _random_state(material)
    h = 1e-6
    fd = (pot.fun(u + h * p) - pot.fun(u - h * p)) / (2 * h)
    assert np.sum(pot.grad(u) * p) == pytest.approx(fd, rel=1e-7)


def test_arap_hess_prod_symmetric_psd():
    """The ARAP Hessian is the reference's PSD approximation (clamped
    lambdas), so it is checked for symmetry and sign rather than by FD."""
    pot, u, p = _random_state(O.Material.ARAP)
    q = np.random.default_rng(7).normal(size=p.shape)
    a = np.sum(pot.hess_prod(u, p) * q)
    b = np.sum(pot.hess_prod(u, q) * p)
    assert a == pytest.approx(b, rel=1e-10)
    pot.clamp_hess_quad = False
    assert np.all(pot.hess_quad_elems(u, p) >= -1e-12)


def test_arap_hess_matches_fd_at_rest_stretch():
    """With all sigma_i + sigma_j >= 2 the clamp is inactive and the ARAP
    Hessian is exact: compare with FD of the gradient."""
    pot, _, p = _random_state(O.Material.ARAP, amp=0.0)
    m = meshgen.grid(3, 3, 2)
    u = 0.2 * m.points  # uniform 20% stretch: sigma = 1.2
    u += 0.002 * np.random.default_rng(3).normal(size=u.shape)
    h = 1e-6
    fd = (pot.grad(u + h * p) - pot.grad(u - h * p)) / (2 * h)
    np.testing.assert_allclose(pot.hess_prod(u, p), fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())


@pytest.mark.parametrize("material", MATERIALS)
def test_hess_quad_equals_p_dot_hess_prod_unclamped(material):
    pot, u, p = _random_state(material, amp=0.02)
    pot.clamp_hess_quad = False
    assert pot.hess_quad(u, p) == pytest.approx(np.sum(pot.hess_prod(u, p) * p), rel=1e-10)


@pytest.mark.parametrize("material", MATERIALS)
def test_hess_diag_equals_assembled_diagonal(material):
    pot, u, _ = _random_state(material, n=(2, 2, 1), amp=0.02)
    pot.clamp_hess_diag = False
    nv = u.shape[0]
    diag = np.zeros((nv, 3))
    for v in range(nv):
        for i in range(3):
            e = np.zeros((nv, 3))
            e[v, i] = 1.0
            diag[v, i] = np.sum(pot.hess_prod(u, e) * e)
    np.testing.assert_allclose(pot.hess_diag(u), diag, rtol=1e-10, atol=1e-12)


def test_snh_hess_prod_fd_exact():
    pot, u, p = _random_state(O.Material.STABLE_NEO_HOOKEAN, seed=3)
    h = 1e-5
    fd = (pot.grad(u + h * p) - pot.grad(u - h * p)) / (2 * h)
    np.testing.assert_allclose(pot.hess_prod(u, p), fd, rtol=1e-6, atol=1e-7 * np.abs(fd).max())


def test_arap_hess_prod_reference_call_order_differs():
    """warp/fem/_arap.py:55-56 swaps (p, dhdX); the intended product differs."""
    pot, u, p = _random_state(O.Material.ARAP)
    F = pot._F(u)
    pc = p[pot.cells]
    a = O.arap_hess_prod(F, pc, pot.dhdX, pot.mu)
    b = O.arap_hess_prod_as_called(F, pc, pot.dhdX, pot.mu)
    assert np.abs(a - b).max() > 1e-3 * np.abs(a).max()


def test_svd_rotation_variant():
    rng = np.random.default_rng(0)
    F = rng.normal(size=(200, 3, 3))
    U, s, V = O.svd_rv(F)
    np.testing.assert_allclose(np.linalg.det(U), 1.0, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(V), 1.0, atol=1e-12)
    np.testing.assert_allclose(np.einsum("nik,nk,njk->nij", U, s, V), F, atol=1e-12)
    assert np.all(np.sign(s[:, 2]) == np.sign(np.linalg.det(F)))
    R, S = O.polar_rv(F)
    np.testing.assert_allclose(R @ S, F, atol=1e-12)


def test_region_rows():
    m = meshgen.grid(2, 2, 2)
    dhdX, dV = O.region_compute_grad(m.points, m.cells)
    np.testing.assert_allclose(dhdX[:, 0], -dhdX[:, 1:].sum(axis=1), atol=1e-12)
    assert dV.sum() == pytest.approx(m.volume())
    # dhdX reproduces a linear field exactly
    A = np.array([[0.1, 0.2, 0.3], [0.0, -0.1, 0.4], [0.2, 0.0, 0.1]])
    u = m.points @ A.T
    F = O.deformation_gradient(u[m.cells], dhdX)
    np.testing.assert_allclose(F, np.broadcast_to(np.eye(3) + A, F.shape), atol=1e-12)


def test_dof_map_roundtrip():
    rng = np.random.default_rng(0)
    mask = rng.random((10, 3)) < 0.3
    fv = rng.normal(size=(10, 3))
    dm = O.DofMap(10, mask, fv)
    free = rng.normal(size=dm.free_indices.size)
    full = dm.to_full(free)
    np.testing.assert_array_equal(full[mask], fv[mask])
    np.testing.assert_array_equal(dm.to_free(full), free)
    assert np.all(dm.to_full_grad(free)[mask] == 0.0)


def test_pncg_separable_quadratic():
    """benches/bench_pncg_branching_backends.py:31-49 objective: with the
    Jacobi preconditioner 1/k the first step is exact."""
    n = 1000
    idx = np.arange(n, dtype=float)
    x0 = np.linspace(-0.9, 0.9, n)
    target = 0.25 * np.sin(idx * 0.001)
    k = 1.0 + np.mod(idx, 17.0) / 17.0
    fun = lambda x: 0.5 * np.sum(k * (x - target) ** 2)  # noqa: E731
    grad = lambda x: k * (x - target)  # noqa: E731
    hd = lambda x: k  # noqa: E731
    hq = lambda x, p: np.sum(k * p * p)  # noqa: E731
    x, st = O.pncg_minimize(fun, grad, hd, hq, x0, rtol=1e-12)
    assert st.result == O.Result.PRIMARY_SUCCESS
    assert st.n_steps == 1
    np.testing.assert_allclose(x, target, atol=1e-12)


def test_snh_small_solve_converges():
    m = meshgen.grid(3, 3, 3)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=mu, lam=lam)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    f = meshgen.lumped_gravity(m, 1000.0)
    ext = O.ExternalForce(np.arange(m.n_points), f)
    model = O.Model(O.DofMap(m.n_points, mask, np.zeros((m.n_points, 3))), [pot], ext)
    u, st = O.solve_model(model, rtol=1e-7, max_steps=2000)
    assert st.result == O.Result.PRIMARY_SUCCESS
    assert u[:, 2].min() < 0.0  # sags under gravity
