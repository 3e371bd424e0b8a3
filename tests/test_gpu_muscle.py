"""Stable Neo-Hookean muscle (G = F A, per-cell activation) on the GPU vs the
FP64 oracle: the five potential methods, the material / activation VJPs,
activation updates, and PNCG solves.

Tolerances: FP64 1e-9 relative; FP32 1e-5 relative L2 (as for the other
materials)."""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-9, torch.float32: 1e-5}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _case(kind, seed=0, amp=0.1):
    rng = np.random.default_rng(seed)
    m = meshgen.grid(5, 4, 6) if kind == "grid" else meshgen.ball(1500, 300, seed=seed)
    nt = m.n_cells
    mu = rng.uniform(0.5, 2.0, nt)
    lam = rng.uniform(1.0, 20.0, nt)
    act = 0.1 * rng.normal(size=(nt, 6))
    X = m.points - m.points.mean(0)
    A = amp * rng.normal(size=(3, 3))
    k = rng.normal(size=(3, 3)) * 2.0
    u = X @ A.T + amp * 0.02 * np.sin(X @ k.T)
    p = X @ rng.normal(size=(3, 3)).T + 0.3 * np.cos(X @ k)
    w = rng.normal(size=u.shape)
    return m, mu, lam, act, u, p, w


def _pots(m, mu, lam, act, dtype):
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.cell_data["mu"] = mu
    mesh.cell_data["lambda"] = lam
    mesh.cell_data["activation"] = act
    gpu = ag.StableNeoHookeanMuscle.from_pyvista(mesh, dtype=dtype)
    ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN_MUSCLE, m.points, m.cells, mu=mu, lam=lam,
                                   activation=act)
    return gpu, ora


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("kind", ["grid", "ball"])
def test_muscle_five_methods_match_oracle(kind, dtype, cuda_device):
    m, mu, lam, act, u, p, _ = _case(kind)
    gpu, ora = _pots(m, mu, lam, act, dtype)
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
    f = gpu.eval(U, Pv, fun=True, grad=True, hess_diag=True, hess_prod=True, hess_quad=True)
    assert f["fun"].item() == pytest.approx(ora.fun(u), rel=tol)
    assert rel_l2(f["grad"].cpu(), ora.grad(u)) < tol
    assert rel_l2(f["hess_prod"].cpu(), ora.hess_prod(u, p)) < tol


def test_muscle_zero_activation_is_stable_neo_hookean(cuda_device):
    dtype = torch.float64
    m, mu, lam, act, u, p, _ = _case("grid", seed=2)
    mus, _ = _pots(m, mu, lam, np.zeros_like(act), dtype)
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.cell_data["mu"] = mu
    mesh.cell_data["lambda"] = lam
    snh = ag.StableNeoHookean.from_pyvista(mesh, dtype=dtype)
    U = torch.tensor(u, dtype=dtype, device=cuda_device)
    Pv = torch.tensor(p, dtype=dtype, device=cuda_device)
    a = mus.eval(U, Pv, fun=True, grad=True, hess_diag=True, hess_prod=True, hess_quad=True)
    b = snh.eval(U, Pv, fun=True, grad=True, hess_diag=True, hess_prod=True, hess_quad=True)
    for k in a:
        np.testing.assert_allclose(a[k].cpu().numpy(), b[k].cpu().numpy(), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_muscle_param_and_activation_vjp(dtype, cuda_device):
    m, mu, lam, act, u, _, w = _case("ball", seed=4)
    gpu, ora = _pots(m, mu, lam, act, dtype)
    U = torch.tensor(u, dtype=dtype, device=cuda_device)
    Wt = torch.tensor(w, dtype=dtype, device=cuda_device)
    out = gpu.grad_param_vjp(U, Wt)
    dmu, dlam = ora.grad_param_vjp(u, w)
    da = ora.grad_activation_vjp(u, w)
    tol = 1e-9 if dtype == torch.float64 else 1e-4
    assert rel_l2(out["mu"].cpu(), dmu) < tol
    assert rel_l2(out["lambda"].cpu(), dlam) < tol
    assert rel_l2(out["activation"].cpu(), da) < tol


def test_set_activation_updates_device_records(cuda_device):
    dtype = torch.float64
    m, mu, lam, act, u, p, _ = _case("grid", seed=5)
    gpu, ora = _pots(m, mu, lam, act, dtype)
    U = torch.tensor(u, dtype=dtype, device=cuda_device)
    g = torch.zeros_like(U)
    gpu.grad(U, g)
    act2 = act[::-1].copy() * 1.5
    gpu.set_activation(act2)
    ora.activation = act2
    g2 = torch.zeros_like(U)
    gpu.grad(U, g2)
    assert rel_l2(g2.cpu(), ora.grad(u)) < 1e-9
    assert rel_l2(g2.cpu(), g.cpu()) > 1e-3


def _muscle_model(dtype, act_scale=-0.15, n=(4, 4, 8)):
    """A column clamped at z = min under gravity; the activation
    (A_zz = 1 + act_scale < 1) makes the rest shape longer along z."""
    m = meshgen.grid(*n)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    nt = m.n_cells
    act = np.zeros((nt, 6))
    act[:, 2] = act_scale
    act[:, 0] = act[:, 1] = -0.5 * act_scale
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mesh.cell_data["activation"] = act
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookeanMuscle.from_pyvista(mesh, dtype=dtype))
    force = meshgen.lumped_gravity(m, 100.0)
    fmesh = meshgen.TetMesh(m.points, m.cells)
    fmesh.point_data["Force"] = force
    fmesh.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fmesh, dtype=dtype))
    pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN_MUSCLE, m.points, m.cells, mu=mu, lam=lam,
                                   activation=act)
    om = O.Model(O.DofMap(m.n_points, mask, fv), [pot], O.ExternalForce(np.arange(m.n_points), force))
    return m, b.finalize(), om


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_muscle_solve_matches_oracle(dtype, cuda_device):
    m, model, om = _muscle_model(dtype)
    rtol = 1e-8 if dtype == torch.float64 else 1e-6
    u_ref, _ = O.solve_model(om, rtol=1e-9, max_steps=5000)
    fwd = ag.Forward(model, ag.PNCG(ag.ConvergenceCriteria(max_steps=5000, rtol=rtol)))
    sol = fwd.step()
    assert sol.result == ag.Result.PRIMARY_SUCCESS, sol
    u = fwd.state.u.double().cpu().numpy()
    diag = np.linalg.norm(m.points.max(0) - m.points.min(0))
    # the activation lengthens the column against gravity (without it the top sags)
    top = meshgen.face_mask(m, 2, "max")
    assert u_ref[top, 2].mean() > 0.03 * m.points[:, 2].max()
    assert np.abs(u - u_ref).max() < 1e-5 * diag


def test_muscle_adjoint_matches_dense_solve(cuda_device):
    """H(u*) lam = r by the device CG on the muscle Hessian (FP64)."""
    m, model, om = _muscle_model(torch.float64, n=(3, 3, 5))
    opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=5000, rtol=1e-10))
    fwd = ag.Forward(model, opt)
    sol = fwd.step()
    assert sol.result == ag.Result.PRIMARY_SUCCESS
    u = fwd.state.u
    dev = opt.solver(fwd.problem)
    rng = np.random.default_rng(0)
    r = rng.normal(size=(m.n_points, 3))
    r[om.dof_map.fixed_mask] = 0.0
    lam_dev, cg = dev.adjoint(torch.tensor(r, dtype=torch.float64, device=cuda_device), rtol=1e-12,
                              max_iter=20000)
    assert cg.result == ag.Result.PRIMARY_SUCCESS
    lam_ref = O.adjoint_dense(om, u.double().cpu().numpy(), r)
    assert rel_l2(lam_dev.cpu(), lam_ref) < 1e-7


def test_activation_gradient_fp64_vs_oracle_and_central_difference(cuda_device):
    """dL/d activation through torch.autograd (the muscle's inverse-fit
    parameter) vs the oracle's implicit gradient and central differences of
    the GPU's FP64 forward (which keeps the resident model between solves)."""
    from apple_gb300.adjoint import EquilibriumFunction, MaterialEquilibrium

    rng = np.random.default_rng(7)
    m = meshgen.grid(3, 3, 6, h=1.0 / 3)
    lam_e, mu_e = meshgen.lame_converter(3e5, 0.4)
    mu = mu_e * rng.uniform(0.5, 2.0, m.n_cells)
    lam = lam_e * np.ones(m.n_cells)
    act = 0.05 * rng.normal(size=(m.n_cells, 6))
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    f = meshgen.lumped_gravity(m, 1000.0)
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    top = meshgen.face_mask(m, 2, "max")
    target = rng.normal(scale=0.01, size=(int(top.sum()), 3))
    crit = ag.ConvergenceCriteria(max_steps=50000, rtol=1e-11)
    prob = MaterialEquilibrium(mesh, ag.StableNeoHookeanMuscle, force=f, dtype=torch.float64, criteria=crit,
                               cg_rtol=1e-11)
    tgt = torch.tensor(target, device=cuda_device)
    topi = torch.tensor(np.flatnonzero(top), device=cuda_device)

    def loss_of(u):
        return 0.5 * ((u[topi] - tgt) ** 2).sum()

    act_t = torch.tensor(act, requires_grad=True)
    u = EquilibriumFunction.apply(torch.tensor(mu), torch.tensor(lam), prob, act_t)
    loss_of(u).backward()
    da = act_t.grad.numpy()
    assert prob.stats.cg.result == ag.Result.PRIMARY_SUCCESS
    ora_pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN_MUSCLE, m.points, m.cells, mu=mu, lam=lam,
                                       activation=act)
    ora_model = O.Model(O.DofMap(m.n_points, mask, np.zeros((m.n_points, 3))), [ora_pot],
                        O.ExternalForce(np.arange(m.n_points), f))
    u64 = u.detach().cpu().numpy()
    dLdu = np.zeros_like(u64)
    dLdu[top] = u64[top] - target
    ref, _ = O.equilibrium_activation_grad(ora_model, ora_pot, u64, dLdu)
    assert rel_l2(da, ref) < 1e-7
    for c, k in ((3, 2), (40, 0), (m.n_cells - 7, 4)):
        h = 1e-5
        vals = []
        for s in (1.0, -1.0):
            a2 = act.copy()
            a2[c, k] += s * h
            vals.append(float(loss_of(prob.solve(torch.tensor(mu), torch.tensor(lam), torch.tensor(a2)))))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert da[c, k] == pytest.approx(fd, rel=1e-4, abs=1e-9 * np.abs(da).max())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_passive_and_muscle_regions_in_one_solve(dtype, cuda_device):
    """A column whose lower half is passive stable Neo-Hookean and whose upper
    half is an activated muscle: two potentials over one vertex set, solved
    by one device PNCG (the passive cells run as muscle cells with zero
    activation) against the oracle's two-potential model."""
    m = meshgen.grid(4, 4, 8)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    zc = m.points[m.cells].mean(1)[:, 2]
    upper = zc > 0.5 * m.points[:, 2].max()
    act = np.zeros((int(upper.sum()), 6))
    act[:, 2] = -0.15
    act[:, 0] = act[:, 1] = 0.075
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    fv = np.zeros((m.n_points, 3))
    force = meshgen.lumped_gravity(m, 100.0)

    def part(sel, muscle):
        mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells[sel]), mu, lam)
        if muscle:
            mesh.cell_data["activation"] = act
        return mesh

    full = meshgen.TetMesh(m.points, m.cells)
    full.point_data["FixedMask"] = mask
    full.point_data["FixedValue"] = fv
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(full)
    b.add_fixed(full)
    b.add_potential(ag.StableNeoHookean.from_pyvista(part(~upper, False), dtype=dtype))
    b.add_potential(ag.StableNeoHookeanMuscle.from_pyvista(part(upper, True), dtype=dtype))
    fmesh = meshgen.TetMesh(m.points, m.cells)
    fmesh.point_data["Force"] = force
    fmesh.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fmesh, dtype=dtype))
    model = b.finalize()
    passive = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells[~upper], mu=mu, lam=lam)
    muscle = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN_MUSCLE, m.points, m.cells[upper], mu=mu,
                                      lam=lam, activation=act)
    om = O.Model(O.DofMap(m.n_points, mask, fv), [passive, muscle], O.ExternalForce(np.arange(m.n_points), force))
    u_ref, _ = O.solve_model(om, rtol=1e-9, max_steps=5000)
    rtol = 1e-8 if dtype == torch.float64 else 1e-6
    fwd = ag.Forward(model, ag.PNCG(ag.ConvergenceCriteria(max_steps=5000, rtol=rtol)))
    sol = fwd.step()
    assert sol.result == ag.Result.PRIMARY_SUCCESS, sol
    fwd_u = fwd.state.u.double().cpu().numpy()
    diag = np.linalg.norm(m.points.max(0) - m.points.min(0))
    assert np.abs(fwd_u - u_ref).max() < 1e-5 * diag
    # the model's own evaluation (per-potential kernels) agrees with the oracle too
    U = torch.tensor(u_ref, dtype=dtype, device=cuda_device)
    g = model.grad(U).double().cpu().numpy()
    g_ref = om.grad(u_ref)
    free = ~mask
    assert np.linalg.norm((g - g_ref)[free]) <= (1e-9 if dtype == torch.float64 else 1e-4) * np.linalg.norm(force)
