"""Batched ARAP (agb_batch_* over ARAP potentials) against the plain
per-model solve and the FP64 oracle (GB300).

ARAP's energy is not polynomial in the step, so its line search needs
element passes: in the batch, the speculative gradient pass at alpha_0 and
its per-mesh Armijo test, then, for the meshes that reject it, the trial
passes and a second gradient pass, each pass returning at once for the
meshes it does not concern.  With overstep 1 most iterations accept alpha_0;
with overstep 4 every one rejects it (on a quadratic model E(4 a*) >
E(2 a*) = E(0) for the Newton step a*), so the iterate tests cover both
branches.  Each model must follow its own Forward.step(): the iteration is
the same, only the reduction order differs.  Bars: FP64 (rtol 1e-10) 1e-7
of the bounding-box diagonal; FP32 (rtol 1e-5, where the plain FP32 ARAP solve
ends too) 1e-4 of it, as for the plain ARAP solve against the oracle."""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from apple_gb300.batch import BatchedForward
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def _case(k, rng):
    """A stretched and twisted ARAP column of uneven size and stiffness."""
    nx, ny, nz = (int(v) for v in rng.integers(2, 6, size=3))
    m = meshgen.grid(nx, ny, nz, h=0.25)
    mu = rng.uniform(0.5, 2.0, m.n_cells)
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.cell_data["mu"] = mu
    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    top = meshgen.face_mask(m, 2, "max")
    mask[top] = True
    zmax = m.points[:, 2].max()
    fv[top, 2] = rng.uniform(0.1, 0.3) * zmax
    c = m.points[top, :2] - m.points[top, :2].mean(0)
    w = rng.uniform(-0.3, 0.3)
    fv[top, 0] = -w * c[:, 1]
    fv[top, 1] = w * c[:, 0]
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    return mesh


def _model(mesh, dtype):
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.Arap.from_pyvista(mesh, dtype=dtype))
    return b.finalize()


def _diag(m):
    return float(np.linalg.norm(m.points.max(0) - m.points.min(0)))


def _opt(rtol, overstep, max_steps=20000):
    return ag.PNCG(ag.ConvergenceCriteria(max_steps=max_steps, rtol=rtol), ag.LineSearch(overstep=overstep))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batch_arap_matches_plain_and_oracle(cuda_device, dtype):
    """Converged solves (overstep 1; with overstep 4 the solve, plain or
    batched, crawls: the first accepted trial is 2 a*, the zero-decrease
    step of a quadratic model)."""
    overstep = 1.0
    rng = np.random.default_rng(11)
    cases = [_case(k, rng) for k in range(5)]
    rtol = 1e-10 if dtype == torch.float64 else 1e-5
    bf = BatchedForward([_model(m, dtype) for m in cases], _opt(rtol, overstep))
    sols, us = bf.solve()
    bar = 1e-7 if dtype == torch.float64 else 1e-4
    for k, (m, sol, u) in enumerate(zip(cases, sols, us)):
        assert sol.result == ag.Result.PRIMARY_SUCCESS, (k, sol)
        assert sol.n_steps > 0
        d = _diag(m)
        fwd = ag.Forward(_model(m, dtype), _opt(rtol, overstep))
        psol = fwd.step()
        assert psol.result == ag.Result.PRIMARY_SUCCESS, (k, psol)
        err_plain = float((u.double() - fwd.state.u.double()).abs().max())
        assert err_plain < bar * d, (k, err_plain / d)
        pot = O.FemPotential.from_mesh(O.Material.ARAP, m.points, m.cells, mu=m.cell_data["mu"])
        om = O.Model(O.DofMap(m.n_points, m.point_data["FixedMask"], m.point_data["FixedValue"]), [pot], None)
        u_ref, _ = O.solve_model(om, rtol=1e-11, max_steps=50000)
        err_ora = float(np.abs(u.double().cpu().numpy() - u_ref).max())
        assert err_ora < bar * d, (k, err_ora / d)


@pytest.mark.parametrize("overstep", [1.0, 4.0])
def test_batch_arap_iterates_follow_plain(cuda_device, overstep):
    """FP64: after 30 iterations every model of the batch is where its own
    solver is after 30 iterations (same Armijo decisions; only the order of
    the global sums differs)."""
    rng = np.random.default_rng(12)
    cases = [_case(k, rng) for k in range(4)]
    bf = BatchedForward([_model(m, torch.float64) for m in cases], _opt(0.0, overstep, 30))
    bf.reset()
    bf.iterate(30)
    sols, us = bf.read()
    for k, (m, sol, u) in enumerate(zip(cases, sols, us)):
        opt = _opt(0.0, overstep, 30)
        fwd = ag.Forward(_model(m, torch.float64), opt)
        sv = opt.solver(fwd.problem)
        sv.reset(fwd.state.u)
        sv.iterate(30)
        up = torch.empty_like(fwd.state.u)
        psol = sv.read(up)
        assert sol.n_steps == psol.n_steps == 30, (k, sol, psol)
        assert float((u.double() - up.double()).abs().max()) < 1e-9 * _diag(m), k


def test_batch_arap_step_and_iterate_agree(cuda_device):
    rng = np.random.default_rng(13)
    cases = [_case(k, rng) for k in range(3)]
    opt = _opt(1e-9, 4.0)
    a = BatchedForward([_model(m, torch.float32) for m in cases], opt)
    a.reset()
    for _ in range(20):
        a.step()
    sa, ua = a.read()
    b = BatchedForward([_model(m, torch.float32) for m in cases], opt)
    b.reset()
    b.iterate(20)
    sb, ub = b.read()
    for x, y, p, q in zip(sa, sb, ua, ub):
        assert x.n_steps == y.n_steps
        assert torch.equal(p, q)  # same kernels, same order: bitwise


def test_batch_rejects_arap_with_stable_neo_hookean(cuda_device):
    rng = np.random.default_rng(14)
    arap = _model(_case(0, rng), torch.float32)
    m, _ = meshgen.batch_case(1, rng, dims=(2, 3), h=0.25)
    b = ag.ModelBuilder(dtype=torch.float32)
    b.add_vertices(m)
    b.add_fixed(m)
    b.add_potential(ag.StableNeoHookean.from_pyvista(m, dtype=torch.float32))
    snh = b.finalize()
    with pytest.raises(RuntimeError, match="cannot share a batch"):
        BatchedForward([arap, snh])
