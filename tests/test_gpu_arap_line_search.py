"""ARAP's line search on the device (GB300): the gradient pass evaluates the
first trial step alpha_0 speculatively and takes its Armijo decision; only a
rejected step runs the trial passes and a second gradient pass.  Each
element's SVD at x is kept between passes.

These tests pin both branches against the FP64 oracle's PNCG
(``oracle/fem_oracle.py`` ``pncg_minimize``, the reference's
``benches/bench_pncg_branching_backends.py:254-456`` loop): with overstep 1
the first trial step is accepted on most iterations; with overstep 4 it is
rejected on every one (on a quadratic model E(4 a*) > E(2 a*) = E(0) for the
Newton step a*), so every iteration goes through the fallback passes."""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def _arap_model(dtype, n=(4, 4, 6), stretch=0.3, seed=0):
    m = meshgen.grid(*n)
    rng = np.random.default_rng(seed)
    mu = rng.uniform(0.5, 2.0, m.n_cells)
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.cell_data["mu"] = mu
    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    top = meshgen.face_mask(m, 2, "max")
    mask[top] = True
    fv[top, 2] = stretch * m.points[:, 2].max()
    # a twist of the top face, so that the rotations change along the solve
    c = m.points[top, :2] - m.points[top, :2].mean(0)
    fv[top, 0] = -0.2 * c[:, 1]
    fv[top, 1] = 0.2 * c[:, 0]
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.Arap.from_pyvista(mesh, dtype=dtype))
    pot = O.FemPotential.from_mesh(O.Material.ARAP, m.points, m.cells, mu=mu)
    om = O.Model(O.DofMap(m.n_points, mask, fv), [pot], None)
    return m, b.finalize(), om


def _solver(model, overstep, max_steps=5000, rtol=0.0):
    opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=max_steps, rtol=rtol), ag.LineSearch(overstep=overstep))
    fwd = ag.Forward(model, opt)
    return fwd, opt.solver(fwd.problem)


@pytest.mark.parametrize("overstep", [1.0, 4.0])
def test_arap_iterates_match_oracle_fp64(overstep, cuda_device):
    """The first iterations follow the oracle's iterate sequence (same Armijo
    decisions, FP64), through the accepted and the rejected branch."""
    m, model, om = _arap_model(torch.float64)
    fwd, dev = _solver(model, overstep, max_steps=100)
    dev.reset(fwd.state.u)
    halvings = []
    done = 0
    for k in (1, 2, 3, 5, 8):
        u_ref, _ = O.solve_model(om, rtol=0.0, max_steps=k, overstep=overstep)
        while done < k:
            dev.iterate(1)
            done += 1
            halvings.append(dev.read().line_search_steps)
        u = torch.empty_like(fwd.state.u)
        s = dev.read(u)
        assert s.n_steps == k
        np.testing.assert_allclose(u.cpu().numpy(), u_ref, rtol=1e-7, atol=1e-10)
    if overstep == 4.0:
        assert min(halvings) >= 1, halvings  # every step came from the fallback passes
    else:
        assert halvings.count(0) >= len(halvings) // 2, halvings


@pytest.mark.parametrize("overstep", [1.0, 4.0])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_arap_solve_matches_oracle(dtype, overstep, cuda_device):
    m, model, om = _arap_model(dtype)
    rtol = 1e-8 if dtype == torch.float64 else 1e-5
    u_ref, _ = O.solve_model(om, rtol=1e-9, max_steps=20000)
    fwd, dev = _solver(model, overstep, rtol=rtol, max_steps=20000)
    dev.reset(fwd.state.u)
    dev.iterate(20000)
    u = torch.empty_like(fwd.state.u)
    s = dev.read(u)
    assert s.result == ag.Result.PRIMARY_SUCCESS, s
    diag = np.linalg.norm(m.points.max(0) - m.points.min(0))
    assert np.abs(u.double().cpu().numpy() - u_ref).max() < 1e-4 * diag


@pytest.mark.parametrize("overstep", [1.0, 4.0])
def test_arap_loop_and_step_graphs_agree(overstep, cuda_device):
    """agb_solver_iterate's loop graph (two iterations per body, the second
    guarded) and the one-iteration step graph give the same bits."""
    m, model, om = _arap_model(torch.float32)
    fwd, dev = _solver(model, overstep)
    dev.reset(fwd.state.u)
    dev.iterate(37)
    u_a = torch.empty_like(fwd.state.u)
    s_a = dev.read(u_a)
    dev.reset(fwd.state.u)
    for _ in range(37):
        dev.step()
    u_b = torch.empty_like(fwd.state.u)
    s_b = dev.read(u_b)
    assert s_a.n_steps == s_b.n_steps == 37
    assert torch.equal(u_a, u_b)
    assert s_a.grad_norm == s_b.grad_norm


def test_arap_checkpoint_resume_is_exact(cuda_device):
    """The checkpoint carries the per-element SVD caches: a restored ARAP
    solve continues bit for bit."""
    m, model, om = _arap_model(torch.float32)
    fwd, dev = _solver(model, 1.0)
    dev.reset(fwd.state.u)
    dev.iterate(8)
    blob = dev.save_state()
    dev.iterate(12)
    u_a = torch.empty_like(fwd.state.u)
    s_a = dev.read(u_a)
    dev.load_state(blob)
    dev.iterate(12)
    u_b = torch.empty_like(fwd.state.u)
    s_b = dev.read(u_b)
    assert s_a.n_steps == s_b.n_steps == 20  # (FP32 reaches its floor near 40 steps on this mesh)
    assert torch.equal(u_a, u_b)
