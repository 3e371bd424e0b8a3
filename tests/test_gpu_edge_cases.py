"""Edge cases of the CUDA path against the FP64 oracle (GB300): a single tet,
an empty potential, vertices that no cell references, per-component fixed
DOFs, the tile-size extremes of the planner, the Fraction scaling of dV, an
inverted tet, and the argument checks of the Python surface.

Tolerances: FP64 1e-9 relative (1e-12 where two device paths must agree),
FP32 1e-5 relative L2."""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _eval_all(pot, u, p, device):
    dt = pot.dtype
    U = torch.tensor(u, dtype=dt, device=device)
    P = torch.tensor(p, dtype=dt, device=device)
    return {k: v.double().cpu().numpy() for k, v in
            pot.eval(U, P, fun=True, grad=True, hess_diag=True, hess_prod=True, hess_quad=True).items()}


def _ora_all(ora, u, p):
    return {"fun": ora.fun(u), "grad": ora.grad(u), "hess_diag": ora.hess_diag(u), "hess_prod": ora.hess_prod(u, p),
            "hess_quad": ora.hess_quad(u, p)}


def _check(got, ref, tol):
    for k in ("fun", "hess_quad"):
        assert float(got[k][0]) == pytest.approx(float(ref[k]), rel=tol, abs=1e-300), k
    for k in ("grad", "hess_diag", "hess_prod"):
        assert rel_l2(got[k], ref[k]) < tol, k


TET = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.2, 0.9, 0.1], [0.1, 0.2, 1.1]])


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("material", ["snh", "arap"])
def test_single_tet(material, dtype, cuda_device):
    rng = np.random.default_rng(0)
    cells = np.array([[0, 1, 2, 3]], np.int32)
    u = 0.05 * rng.normal(size=(4, 3))
    p = rng.normal(size=(4, 3))
    if material == "snh":
        pot = ag.StableNeoHookean(cells, 2.0, 7.0, points=TET, dtype=dtype)
        ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, TET, cells, mu=2.0, lam=7.0)
    else:
        pot = ag.Arap(cells, 2.0, points=TET, dtype=dtype)
        ora = O.FemPotential.from_mesh(O.Material.ARAP, TET, cells, mu=2.0)
    _check(_eval_all(pot, u, p, cuda_device), _ora_all(ora, u, p), 1e-9 if dtype == torch.float64 else 1e-5)


def test_empty_potential_leaves_outputs_alone(cuda_device):
    cells = np.zeros((0, 4), np.int32)
    pot = ag.StableNeoHookean(cells, np.zeros(0), np.zeros(0), points=TET, n_points=4, dtype=torch.float64)
    U = torch.zeros((4, 3), dtype=torch.float64, device=cuda_device)
    out = torch.full((1,), 3.0, dtype=torch.float64, device=cuda_device)
    pot.fun(U, out)
    assert out.item() == 3.0
    g = torch.full((4, 3), 2.0, dtype=torch.float64, device=cuda_device)
    pot.grad(U, g)
    pot.hess_diag(U, g)
    pot.hess_prod(U, U, g)
    assert torch.all(g == 2.0)
    q = torch.full((1,), 5.0, dtype=torch.float64, device=cuda_device)
    pot.hess_quad(U, U, q)
    assert q.item() == 5.0


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_isolated_vertices_and_per_component_fixed_dofs(dtype, cuda_device):
    """Points that no cell references stay where they are; a face fixed in z
    only slides in x and y."""
    m = meshgen.grid(3, 3, 4)
    extra = np.array([[5.0, 5.0, 5.0], [6.0, 5.0, 5.0]])
    pts = np.concatenate([m.points, extra])
    n = pts.shape[0]
    lam, mu = meshgen.lame_converter(1e4, 0.4)
    mesh = ag.with_lame(meshgen.TetMesh(pts, m.cells), mu, lam)
    mask = np.zeros((n, 3), bool)
    fv = np.zeros((n, 3))
    bottom = np.zeros(n, bool)
    bottom[: m.n_points] = meshgen.face_mask(m, 2, "min")
    top = np.zeros(n, bool)
    top[: m.n_points] = meshgen.face_mask(m, 2, "max")
    mask[bottom] = True
    mask[top, 2] = True  # z only
    fv[top, 2] = 0.1
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, dtype=dtype))
    model = b.finalize()
    rtol = 1e-10 if dtype == torch.float64 else 1e-6
    fwd = ag.Forward(model, ag.PNCG(ag.ConvergenceCriteria(max_steps=5000, rtol=rtol)))
    sol = fwd.step()
    assert sol.result == ag.Result.PRIMARY_SUCCESS, sol
    u = fwd.state.u.double().cpu().numpy()
    pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, pts, m.cells, mu=mu, lam=lam)
    om = O.Model(O.DofMap(n, mask, fv), [pot], None)
    u_ref, _ = O.solve_model(om, rtol=1e-10, max_steps=5000)
    np.testing.assert_array_equal(u[-2:], 0.0)
    np.testing.assert_allclose(u[top, 2], 0.1, rtol=0, atol=1e-7)
    assert np.abs(u[top, :2]).max() > 1e-4  # the z-only face slides sideways (Poisson contraction)
    diag = np.linalg.norm(m.points.max(0) - m.points.min(0))
    assert np.abs(u - u_ref).max() < (1e-6 if dtype == torch.float64 else 1e-4) * diag


def test_tile_size_extremes_agree(cuda_device):
    """One element per tile, 32 per tile and the 1024 default give the same
    values (FP64; only the summation order differs)."""
    rng = np.random.default_rng(3)
    m = meshgen.ball(400, 100, seed=3)
    mu = rng.uniform(0.5, 2.0, m.n_cells)
    lam = rng.uniform(1.0, 20.0, m.n_cells)
    X = m.points - m.points.mean(0)
    u = X @ (0.05 * rng.normal(size=(3, 3))).T
    p = rng.normal(size=u.shape)
    outs = []
    for te in (1, 32, 0):
        pot = ag.StableNeoHookean(m.cells, mu, lam, points=m.points, dtype=torch.float64, tile_elems=te)
        outs.append(_eval_all(pot, u, p, cuda_device))
    for o in outs[:2]:
        for k in o:
            np.testing.assert_allclose(o[k], outs[2][k], rtol=1e-12, atol=1e-12 * np.abs(outs[2][k]).max())


def test_fraction_scales_the_volume(cuda_device):
    rng = np.random.default_rng(4)
    m = meshgen.grid(4, 3, 3)
    frac = rng.uniform(0.2, 1.0, m.n_cells)
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.cell_data["mu"] = np.full(m.n_cells, 1.5)
    mesh.cell_data["lambda"] = np.full(m.n_cells, 9.0)
    mesh.cell_data["Fraction"] = frac
    pot = ag.StableNeoHookean.from_pyvista(mesh, dtype=torch.float64)
    ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=1.5, lam=9.0, fraction=frac)
    u = 0.03 * rng.normal(size=(m.n_points, 3))
    p = rng.normal(size=u.shape)
    _check(_eval_all(pot, u, p, cuda_device), _ora_all(ora, u, p), 1e-9)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_inverted_tet_stable_neo_hookean(dtype, cuda_device):
    """Stable Neo-Hookean is defined through inversion (J < 0)."""
    cells = np.array([[0, 1, 2, 3]], np.int32)
    u = np.zeros((4, 3))
    u[3] = [0.0, 0.0, -1.6]  # pushes the apex through the base: J < 0
    p = np.random.default_rng(5).normal(size=(4, 3))
    ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, TET, cells, mu=2.0, lam=7.0)
    F = O.deformation_gradient(u[cells], ora.dhdX)
    assert np.linalg.det(F)[0] < 0
    pot = ag.StableNeoHookean(cells, 2.0, 7.0, points=TET, dtype=dtype)
    _check(_eval_all(pot, u, p, cuda_device), _ora_all(ora, u, p), 1e-9 if dtype == torch.float64 else 1e-5)


def test_argument_checks(cuda_device):
    cells = np.array([[0, 1, 2, 3]], np.int32)
    pot = ag.StableNeoHookean(cells, 2.0, 7.0, points=TET, dtype=torch.float32)
    out = torch.zeros((4, 3), dtype=torch.float32, device=cuda_device)
    with pytest.raises(TypeError):
        pot.grad(torch.zeros((4, 3), dtype=torch.float64, device=cuda_device), out)
    with pytest.raises(TypeError):
        pot.grad(torch.zeros((4, 3), dtype=torch.float32), out)
    with pytest.raises(ValueError):
        pot.grad(torch.zeros((5, 3), dtype=torch.float32, device=cuda_device), out)
    with pytest.raises(ValueError):
        pot.grad(torch.zeros((3, 4), dtype=torch.float32, device=cuda_device).t(), out)
    with pytest.raises(TypeError):
        pot.fun(torch.zeros((4, 3), dtype=torch.float32, device=cuda_device),
                torch.zeros(1, dtype=torch.float32, device=cuda_device))


def _tet_displacement_for(F):
    """u with deformation gradient F on TET (u_a = (F - I) X_a)."""
    return (TET - TET[0]) @ (np.asarray(F) - np.eye(3)).T


@pytest.mark.parametrize("case", ["inverted", "rotation", "repeated_singular_values", "near_flat"])
def test_arap_svd_edge_cases_fp64(case, cuda_device):
    """ARAP at deformation gradients where the 3x3 SVD is delicate: an
    inverted tet (rotation-variant convention, det R = +1), a pure rotation
    (zero energy and force), repeated singular values (R unique although U
    and V are not), and a nearly flat tet."""
    cells = np.array([[0, 1, 2, 3]], np.int32)
    c, s_ = np.cos(0.7), np.sin(0.7)
    Rz = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
    F = {"inverted": np.diag([1.1, 0.9, -0.8]) @ Rz,
         "rotation": Rz,
         "repeated_singular_values": Rz @ np.diag([1.2, 1.2, 0.9]),
         "near_flat": np.diag([1.0, 1.0, 1e-3]) @ Rz}[case]
    u = _tet_displacement_for(F)
    p = np.random.default_rng(6).normal(size=(4, 3))
    ora = O.FemPotential.from_mesh(O.Material.ARAP, TET, cells, mu=2.0)
    pot = ag.Arap(cells, 2.0, points=TET, dtype=torch.float64)
    got = _eval_all(pot, u, p, cuda_device)
    ref = _ora_all(ora, u, p)
    if case == "rotation":
        assert abs(float(got["fun"][0])) < 1e-12 and np.abs(got["grad"]).max() < 1e-12
        return
    _check(got, ref, 1e-9)
