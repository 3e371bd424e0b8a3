"""CUDA path vs the FP64 oracle on the same seeded inputs (GB300).

Tolerances: FP64 kernels 1e-9 relative; FP32 kernels 1e-5 relative L2 for
energy, gradient, Hessian diagonal and products (the stated parity bar for
FP32 element math with float-float/FP64 reductions)."""

import json
import pathlib

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).parent / "golden"
TOL = {torch.float64: 1e-9, torch.float32: 1e-5}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _case(material, kind, seed=0, amp=0.1):
    rng = np.random.default_rng(seed)
    m = meshgen.grid(5, 4, 6) if kind == "grid" else meshgen.ball(1500, 300, seed=seed)
    nt = m.n_cells
    mu = rng.uniform(0.5, 2.0, nt)
    lam = rng.uniform(1.0, 20.0, nt) if material == "snh" else None
    # smooth field (bounded strain on the sliver tets of a Delaunay mesh)
    X = m.points - m.points.mean(0)
    A = amp * rng.normal(size=(3, 3))
    k = rng.normal(size=(3, 3)) * 2.0
    u = X @ A.T + amp * 0.02 * np.sin(X @ k.T)
    p = X @ rng.normal(size=(3, 3)).T + 0.3 * np.cos(X @ k)
    return m, mu, lam, u, p


def _pots(material, m, mu, lam, dtype):
    cls = ag.Arap if material == "arap" else ag.StableNeoHookean
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.cell_data["mu"] = mu
    if lam is not None:
        mesh.cell_data["lambda"] = lam
    gpu = cls.from_pyvista(mesh, dtype=dtype)
    mat = O.Material.ARAP if material == "arap" else O.Material.STABLE_NEO_HOOKEAN
    ora = O.FemPotential.from_mesh(mat, m.points, m.cells, mu=mu, lam=lam)
    return gpu, ora


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("material", ["snh", "arap"])
@pytest.mark.parametrize("kind", ["grid", "ball"])
def test_five_methods_match_oracle(material, kind, dtype, cuda_device):
    m, mu, lam, u, p = _case(material, kind)
    gpu, ora = _pots(material, m, mu, lam, dtype)
    U = torch.tensor(u, dtype=dtype, device=cuda_device)
    Pv = torch.tensor(p, dtype=dtype, device=cuda_device)
    tol = TOL[dtype]
    out = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    gpu.fun(U, out)
    assert out.item() == pytest.approx(ora.fun(u), rel=tol)
    g = torch.zeros_like(U)
    gpu.grad(U, g)
    assert rel_l2(g.cpu(), ora.grad(u)) < tol
    d = torch.zeros_like(U)
    gpu.hess_diag(U, d)
    assert rel_l2(d.cpu(), ora.hess_diag(u)) < tol
    hp = torch.zeros_like(U)
    gpu.hess_prod(U, Pv, hp)
    assert rel_l2(hp.cpu(), ora.hess_prod(u, p)) < tol
    q = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    gpu.hess_quad(U, Pv, q)
    assert q.item() == pytest.approx(ora.hess_quad(u, p), rel=tol)


@pytest.mark.parametrize("material", ["snh", "arap"])
def test_outputs_accumulate_and_fused_matches_separate(material, cuda_device):
    dtype = torch.float64
    m, mu, lam, u, p = _case(material, "grid", seed=1)
    gpu, ora = _pots(material, m, mu, lam, dtype)
    U = torch.tensor(u, dtype=dtype, device=cuda_device)
    Pv = torch.tensor(p, dtype=dtype, device=cuda_device)
    g = torch.ones_like(U)
    gpu.grad(U, g)
    np.testing.assert_allclose(g.cpu().numpy() - 1.0, ora.grad(u), rtol=1e-9, atol=1e-12)
    e = torch.full((1,), 2.0, dtype=torch.float64, device=cuda_device)
    gpu.fun(U, e)
    assert e.item() - 2.0 == pytest.approx(ora.fun(u), rel=1e-9)
    f = gpu.eval(U, Pv, fun=True, grad=True, hess_diag=True, hess_prod=True, hess_quad=True)
    assert f["fun"].item() == pytest.approx(ora.fun(u), rel=1e-9)
    assert rel_l2(f["grad"].cpu(), ora.grad(u)) < 1e-9
    assert rel_l2(f["hess_diag"].cpu(), ora.hess_diag(u)) < 1e-9
    assert rel_l2(f["hess_prod"].cpu(), ora.hess_prod(u, p)) < 1e-9
    assert f["hess_quad"].item() == pytest.approx(ora.hess_quad(u, p), rel=1e-9)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_model_with_fixed_and_force(dtype, cuda_device):
    m = meshgen.grid(4, 4, 4)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, dtype=dtype))
    force = meshgen.lumped_gravity(m, 1000.0)
    fmesh = meshgen.TetMesh(m.points, m.cells)
    fmesh.point_data["Force"] = force
    fmesh.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fmesh, dtype=dtype))
    model = b.finalize()
    pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=mu, lam=lam)
    om = O.Model(O.DofMap(m.n_points, mask, np.zeros((m.n_points, 3))), [pot],
                 O.ExternalForce(np.arange(m.n_points), force))
    u = 0.01 * np.random.default_rng(0).normal(size=(m.n_points, 3))
    U = torch.tensor(u, dtype=dtype, device=cuda_device)
    tol = TOL[dtype]
    assert model.fun(U).item() == pytest.approx(om.fun(u), rel=tol)
    assert rel_l2(model.grad(U).cpu(), om.grad(u)) < tol
    assert rel_l2(model.hess_diag(U).cpu(), om.hess_diag(u)) < tol


def _embedded(dtype):
    d = json.loads((GOLDEN / "embedded_tetra.json").read_text())
    mesh = meshgen.TetMesh(np.asarray(d["points"], float), np.asarray(d["cells"], np.int32))
    mesh.cell_data["mu"] = np.full(len(d["cells"]), d["mu"])
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    mask = np.zeros((len(d["points"]), 3), bool)
    mask[d["fixed_vertices"]] = True
    fv = np.zeros((len(d["points"]), 3))
    fv[d["fixed_value_vertex"]] = d["fixed_value"]
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    b.add_fixed(mesh)
    b.add_potential(ag.Arap.from_pyvista(mesh, dtype=dtype))
    return d, b.finalize(), fv


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_embedded_vertex_known_answer(dtype, cuda_device):
    """tests/forward/test_static_simulation.py:58-93 of the reference."""
    d, model, fv = _embedded(dtype)
    fwd = ag.Forward(model)
    e0 = float(fwd.problem.fun(fwd.state))
    sol = fwd.step()
    e1 = float(fwd.problem.fun(fwd.state))
    u = fwd.state.u.double().cpu().numpy()
    assert model.n_free == d["n_free"]
    assert np.isfinite(e0) and np.isfinite(e1) and e1 < e0
    np.testing.assert_allclose(u[:4], fv[:4])
    atol = d["atol"] if dtype == torch.float64 else 1e-6
    if dtype == torch.float64:
        assert sol.result.name == d["result"]
    np.testing.assert_allclose(u[d["expect_vertex"]], d["expect_u"], atol=atol)


def _snh_model(dtype, n=(4, 4, 6), gravity=True, stretch=False):
    m = meshgen.grid(*n)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    if stretch:
        top = meshgen.face_mask(m, 2, "max")
        mask[top] = True
        fv[top, 2] = 0.3 * m.points[:, 2].max()
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, dtype=dtype))
    force = meshgen.lumped_gravity(m, 1000.0) if gravity else None
    if gravity:
        fmesh = meshgen.TetMesh(m.points, m.cells)
        fmesh.point_data["Force"] = force
        fmesh.point_data["GlobalPointId"] = np.arange(m.n_points)
        b.add_potential(ag.ExternalForce.from_pyvista(fmesh, dtype=dtype))
    pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=mu, lam=lam)
    om = O.Model(O.DofMap(m.n_points, mask, fv), [pot],
                 O.ExternalForce(np.arange(m.n_points), force) if gravity else None)
    return m, b.finalize(), om


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("stretch", [False, True])
def test_snh_solve_matches_oracle(dtype, stretch, cuda_device):
    m, model, om = _snh_model(dtype, gravity=not stretch, stretch=stretch)
    rtol = 1e-8 if dtype == torch.float64 else 1e-5
    u_ref, st_ref = O.solve_model(om, rtol=1e-9, max_steps=5000)
    fwd = ag.Forward(model, ag.PNCG(ag.ConvergenceCriteria(max_steps=5000, rtol=rtol)))
    sol = fwd.step()
    assert sol.result == ag.Result.PRIMARY_SUCCESS, sol
    u = fwd.state.u.double().cpu().numpy()
    diag = np.linalg.norm(m.points.max(0) - m.points.min(0))
    assert np.abs(u - u_ref).max() < 1e-4 * diag


def test_pncg_iterates_match_oracle_fp64(cuda_device):
    """First iterations of the device PNCG follow the oracle's iterate
    sequence (same Armijo decisions, FP64 everywhere)."""
    m, model, om = _snh_model(torch.float64, gravity=True)
    dm = om.dof_map
    xs = []
    for k in (1, 2, 3, 5, 8):
        u_ref, st = O.solve_model(om, rtol=0.0, max_steps=k)
        xs.append((k, u_ref, st))
    solver = ag.PNCG(ag.ConvergenceCriteria(max_steps=100, rtol=0.0))
    fwd = ag.Forward(model, solver)
    dev = solver.solver(fwd.problem)
    dev.reset(fwd.state.u)
    done = 0
    for k, u_ref, st in xs:
        dev.iterate(k - done)
        done = k
        u = torch.empty_like(fwd.state.u)
        s = dev.read(u)
        assert s.n_steps == k
        np.testing.assert_allclose(u.cpu().numpy(), u_ref, rtol=1e-7, atol=1e-10)
    del dm


def test_solver_step_graph_and_host_minimize(cuda_device):
    m, model, om = _snh_model(torch.float32, gravity=True)
    solver = ag.PNCG(ag.ConvergenceCriteria(max_steps=400, rtol=1e-5))
    fwd = ag.Forward(model, solver)
    dev = solver.solver(fwd.problem)
    dev.reset(fwd.state.u)
    for _ in range(5):
        dev.step()
    s = dev.read()
    assert s.n_steps == 5
    u_host = fwd.state.u.cpu().clone()
    sol = dev.minimize_host(u_host)
    assert sol.result == ag.Result.PRIMARY_SUCCESS
    u_ref, _ = O.solve_model(om, rtol=1e-9, max_steps=5000)
    diag = np.linalg.norm(m.points.max(0) - m.points.min(0))
    assert np.abs(u_host.double().numpy() - u_ref).max() < 1e-4 * diag


def test_stored_connectivity_is_exact_and_deterministic(cuda_device):
    """Morton reorder + tiling + warp-group colouring keep every cell's corner
    set, and building the plan twice gives the same plan (bit-exact)."""
    m = meshgen.ball(1500, 300, seed=3)
    rng = np.random.default_rng(3)
    perm = rng.permutation(m.n_points)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(m.n_points)
    pts, cells = m.points[perm], inv[m.cells].astype(np.int32)
    mu = np.ones(cells.shape[0])
    a = ag.StableNeoHookean(cells, mu, 10 * mu, points=pts)
    b = ag.StableNeoHookean(cells, mu, 10 * mu, points=pts)
    ca, ha = a.stored_cells()
    cb, hb = b.stored_cells()
    assert np.array_equal(np.sort(ca, axis=1), np.sort(cells, axis=1))
    assert np.array_equal(ca, cb) and ha == hb
