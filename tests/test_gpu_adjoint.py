"""Adjoint of the equilibrium on the GPU against the FP64 oracle (GB300).

- the material VJP of the gradient (agb_fem_grad_param_vjp) vs the oracle's;
- the device CG (agb_solver_adjoint) vs a dense FP64 solve at the same u*;
- dL/dmu through torch.autograd (EquilibriumFunction) vs the oracle's implicit
  gradient and vs central differences of the GPU's own FP64 forward.
Tolerances are written per test."""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from apple_gb300.adjoint import EquilibriumFunction, MaterialEquilibrium
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("material", ["snh", "arap"])
def test_grad_param_vjp_matches_oracle(cuda_device, material, dtype):
    rng = np.random.default_rng(11)
    m = meshgen.grid(5, 4, 6)
    mu = rng.uniform(0.5, 2.0, m.n_cells)
    lam = rng.uniform(1.0, 20.0, m.n_cells) if material == "snh" else None
    u = 0.05 * rng.normal(size=(m.n_points, 3))
    w = rng.normal(size=(m.n_points, 3))
    cls = ag.StableNeoHookean if material == "snh" else ag.Arap
    pot = cls(m.cells, mu, lam, points=m.points, dtype=dtype)
    out = pot.grad_param_vjp(torch.tensor(u, dtype=dtype, device=cuda_device),
                             torch.tensor(w, dtype=dtype, device=cuda_device))
    ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN if material == "snh" else O.Material.ARAP,
                                   m.points, m.cells, mu=mu, lam=lam)
    dmu, dlam = ora.grad_param_vjp(u, w)
    tol = 1e-10 if dtype == torch.float64 else 1e-5
    assert rel_l2(out["mu"].cpu(), dmu) < tol
    if material == "snh":
        assert rel_l2(out["lambda"].cpu(), dlam) < tol
    else:
        assert "lambda" not in out


def _gravity_column(dtype, seed=5):
    rng = np.random.default_rng(seed)
    m = meshgen.grid(3, 3, 6, h=1.0 / 3)
    lam_e, mu_e = meshgen.lame_converter(3e5, 0.4)
    mu = mu_e * rng.uniform(0.5, 2.0, m.n_cells)
    lam = lam_e * np.ones(m.n_cells)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    f = meshgen.lumped_gravity(m, 1000.0)
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    top = meshgen.face_mask(m, 2, "max")
    target = rng.normal(scale=0.01, size=(int(top.sum()), 3))
    crit = ag.ConvergenceCriteria(max_steps=50000, rtol=1e-11 if dtype == torch.float64 else 1e-6)
    prob = MaterialEquilibrium(mesh, ag.StableNeoHookean, force=f, dtype=dtype, criteria=crit,
                               cg_rtol=1e-11 if dtype == torch.float64 else 1e-6)
    ora_pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=mu, lam=lam)
    ora_model = O.Model(O.DofMap(m.n_points, mask, np.zeros((m.n_points, 3))), [ora_pot],
                        O.ExternalForce(np.arange(m.n_points), f))
    return m, mu, lam, top, target, prob, ora_pot, ora_model


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_adjoint_cg_matches_dense_solve(cuda_device, dtype):
    m, mu, lam, top, target, prob, ora_pot, ora_model = _gravity_column(dtype)
    u = prob.solve(torch.tensor(mu), torch.tensor(lam))
    assert prob.stats.forward.result == ag.Result.PRIMARY_SUCCESS
    rng = np.random.default_rng(1)
    rhs = rng.normal(size=(m.n_points, 3))
    _, sv, u_dev, _ = prob._state
    lam_gpu, cg = sv.adjoint(torch.tensor(rhs, dtype=dtype, device=cuda_device),
                             rtol=1e-11 if dtype == torch.float64 else 1e-6)
    assert cg.result == ag.Result.PRIMARY_SUCCESS, cg
    u64 = u_dev.double().cpu().numpy()
    ref = O.adjoint_dense(ora_model, u64, rhs)
    lam_np = lam_gpu.double().cpu().numpy()
    assert np.all(lam_np[ora_model.dof_map.fixed_mask] == 0.0)
    assert rel_l2(lam_np, ref) < (1e-8 if dtype == torch.float64 else 2e-4)


def test_equilibrium_gradient_fp64_vs_oracle_and_central_difference(cuda_device):
    dtype = torch.float64
    m, mu, lam, top, target, prob, ora_pot, ora_model = _gravity_column(dtype)
    mu_t = torch.tensor(mu, requires_grad=True)
    lam_t = torch.tensor(lam, requires_grad=True)
    tgt = torch.tensor(target, device=cuda_device)
    topi = torch.tensor(np.flatnonzero(top), device=cuda_device)

    def loss_of(u):
        return 0.5 * ((u[topi] - tgt) ** 2).sum()

    u = EquilibriumFunction.apply(mu_t, lam_t, prob)
    L = loss_of(u)
    L.backward()
    dmu = mu_t.grad.numpy()
    dlam = lam_t.grad.numpy()
    assert prob.stats.cg.result == ag.Result.PRIMARY_SUCCESS
    # the oracle's implicit gradient at the GPU's u*
    u64 = u.detach().cpu().numpy()
    dLdu = np.zeros_like(u64)
    dLdu[top] = u64[top] - target
    ref_mu, ref_lam, _ = O.equilibrium_param_grad(ora_model, ora_pot, u64, dLdu)
    assert rel_l2(dmu, ref_mu) < 1e-7
    assert rel_l2(dlam, ref_lam) < 1e-7
    # central differences of the GPU forward (h = 1e-4 relative) on a few cells
    for c in (2, 77, m.n_cells - 5):
        h = 1e-4 * mu[c]
        vals = []
        for s in (1.0, -1.0):
            mu2 = mu.copy()
            mu2[c] += s * h
            vals.append(float(loss_of(prob.solve(torch.tensor(mu2), torch.tensor(lam)))))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert dmu[c] == pytest.approx(fd, rel=1e-5)


def test_equilibrium_gradient_fp32_vs_fp64_oracle(cuda_device):
    dtype = torch.float32
    m, mu, lam, top, target, prob, ora_pot, ora_model = _gravity_column(dtype)
    mu_t = torch.tensor(mu, requires_grad=True)
    tgt = torch.tensor(target, dtype=torch.float32, device=cuda_device)
    topi = torch.tensor(np.flatnonzero(top), device=cuda_device)
    u = EquilibriumFunction.apply(mu_t, torch.tensor(lam), prob)
    (0.5 * ((u.float()[topi] - tgt) ** 2).sum()).backward()
    # FP64 oracle: forward to 1e-9, implicit gradient at its own u*
    u_ref, _ = O.solve_model(ora_model, rtol=1e-10, max_steps=20000)
    dLdu = np.zeros_like(u_ref)
    dLdu[top] = u_ref[top] - target
    ref_mu, _, _ = O.equilibrium_param_grad(ora_model, ora_pot, u_ref, dLdu)
    assert rel_l2(mu_t.grad.numpy(), ref_mu) < 5e-3
