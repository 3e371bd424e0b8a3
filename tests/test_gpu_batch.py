"""Batched PNCG (agb_batch_*) against the plain per-model solve and the FP64
oracle (GB300).  Each model of the batch must converge to the displacement
its own Forward.step() gives: the iteration is the same, only the reduction
order differs.  Bars: FP64 (rtol 1e-10) 1e-7 of the bounding-box diagonal vs
the plain solve and vs the oracle; FP32 (rtol 1e-6, with the reference-state
correction) 1e-5 of the diagonal."""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from apple_gb300.batch import BatchedForward, autotune
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def _model(m, f, dtype, tile_elems=0):
    pot = ag.StableNeoHookean.from_pyvista(m, dtype=dtype, tile_elems=tile_elems)
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(m)
    b.add_fixed(m)
    b.add_potential(pot)
    fm = meshgen.TetMesh(m.points, m.cells)
    fm.point_data["Force"] = f
    fm.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fm, dtype=dtype))
    return b.finalize()


def _cases(n, seed=0, dims=(2, 6)):
    rng = np.random.default_rng(seed)
    return [meshgen.batch_case(k, rng, dims=dims, h=0.25) for k in range(n)]


def _diag(m):
    return float(np.linalg.norm(m.points.max(0) - m.points.min(0)))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batch_matches_plain_and_oracle(cuda_device, dtype):
    cases = _cases(7)
    rtol = 1e-10 if dtype == torch.float64 else 1e-6
    crit = ag.ConvergenceCriteria(max_steps=20000, rtol=rtol)
    models = [_model(m, f, dtype) for m, f in cases]
    bf = BatchedForward(models, ag.PNCG(crit))
    sols, us = bf.solve()
    for k, ((m, f), sol, u) in enumerate(zip(cases, sols, us)):
        assert sol.result == ag.Result.PRIMARY_SUCCESS, (k, sol)
        d = _diag(m)
        # the plain per-model solve
        fwd = ag.Forward(_model(m, f, dtype), ag.PNCG(crit))
        psol = fwd.step()
        assert psol.result == ag.Result.PRIMARY_SUCCESS
        # the preconditioner's diagonal mean at (nearly) the same equilibrium
        assert sol.hess_diag_mean > 0 and abs(sol.hess_diag_mean / psol.hess_diag_mean - 1) < 1e-3
        err_plain = float((u.double() - fwd.state.u.double()).abs().max())
        # the FP64 oracle
        ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells,
                                       mu=m.cell_data["mu"], lam=m.cell_data["lambda"])
        om = O.Model(O.DofMap(m.n_points, m.point_data["FixedMask"], np.zeros((m.n_points, 3))), [ora],
                     O.ExternalForce(np.arange(m.n_points), f))
        u_ref, _ = O.solve_model(om, rtol=1e-11, max_steps=50000)
        err_ora = float(np.abs(u.double().cpu().numpy() - u_ref).max())
        if dtype == torch.float64:
            assert err_plain < 1e-7 * d, (k, err_plain)
            assert err_ora < 1e-7 * d, (k, err_ora)
        else:
            assert err_plain < 1e-5 * d, (k, err_plain)
            assert err_ora < 1e-5 * d, (k, err_ora)
        assert sol.n_steps > 0


def test_batch_step_and_iterate_agree(cuda_device):
    cases = _cases(4, seed=3)
    crit = ag.ConvergenceCriteria(max_steps=20000, rtol=1e-9)
    models = [_model(m, f, torch.float64) for m, f in cases]
    a = BatchedForward(models, ag.PNCG(crit))
    a.reset()
    for _ in range(25):
        a.step()
    sa, ua = a.read()
    b = BatchedForward(models, ag.PNCG(crit))
    b.reset()
    b.iterate(25)
    sb, ub = b.read()
    for x, y, p, q in zip(sa, sb, ua, ub):
        assert x.n_steps == y.n_steps
        assert torch.equal(p, q)  # same kernels, same order: bitwise


def test_autotuner_picks_a_candidate(cuda_device):
    cases = _cases(3, seed=5)
    res = autotune(lambda te: [_model(m, f, torch.float32, tile_elems=te) for m, f in cases],
                   tile_elems=(256, 1024), chunk_verts=(256, 512), iters=3)
    assert (res.tile_elems, res.chunk_verts) in [(t, c) for t, c, _ in res.table]
    assert res.ms_per_iter == min(ms for _, _, ms in res.table)


def _muscle_model(m, f, dtype, act):
    mm = meshgen.TetMesh(m.points, m.cells)
    mm.cell_data.update(m.cell_data)
    mm.point_data.update(m.point_data)
    mm.cell_data["activation"] = act
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mm)
    b.add_fixed(mm)
    b.add_potential(ag.StableNeoHookeanMuscle.from_pyvista(mm, dtype=dtype))
    fm = meshgen.TetMesh(m.points, m.cells)
    fm.point_data["Force"] = f
    fm.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fm, dtype=dtype))
    return b.finalize()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batch_with_muscle_models(cuda_device, dtype):
    """Stable Neo-Hookean and activated muscle models in one batch (all cells
    run as muscle cells, the plain ones with zero activation): each model
    follows its own plain solve."""
    cases = _cases(5, seed=3)
    rng = np.random.default_rng(4)
    acts = {1: 0.05 * rng.normal(size=(cases[1][0].n_cells, 6)), 3: 0.05 * rng.normal(size=(cases[3][0].n_cells, 6))}
    rtol = 1e-10 if dtype == torch.float64 else 1e-6
    crit = ag.ConvergenceCriteria(max_steps=20000, rtol=rtol)

    def build(k):
        m, f = cases[k]
        return _muscle_model(m, f, dtype, acts[k]) if k in acts else _model(m, f, dtype)

    bf = BatchedForward([build(k) for k in range(len(cases))], ag.PNCG(crit))
    sols, us = bf.solve()
    bar = 1e-7 if dtype == torch.float64 else 1e-5
    for k, (sol, u) in enumerate(zip(sols, us)):
        assert sol.result == ag.Result.PRIMARY_SUCCESS, (k, sol)
        fwd = ag.Forward(build(k), ag.PNCG(crit))
        assert fwd.step().result == ag.Result.PRIMARY_SUCCESS
        assert float((u.double() - fwd.state.u.double()).abs().max()) < bar * _diag(cases[k][0]), k
