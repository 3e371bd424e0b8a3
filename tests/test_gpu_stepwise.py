"""Step-by-step driving of the device PNCG (``PNCG.init / step / terminate /
postprocess``, as the loop of exp/2026/05/06/toy/src/
20-ext-force-stable-neo-hookean-collision.py:236-251 drives it) and the
optimizer state that loop's progress logging reads (lines 207-233): the line-search
and convergence states, the search direction and the Hessian-diagonal mean
(GB300).

At u = 0 the elements carry no stress, so the first gradient is -f exactly
and the first direction is f / |diag|; every accepted step moves the free
DOFs by alpha * direction; the stepped solve ends where the one-call solve
ends."""

import math

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _column(dtype, n=(4, 4, 6)):
    m = meshgen.grid(*n)
    lam, mu = meshgen.lame_converter(1e5, 0.45)
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, dtype=dtype))
    fm = meshgen.TetMesh(m.points, m.cells)
    fm.point_data["Force"] = meshgen.lumped_gravity(m, 1000.0)
    fm.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fm, dtype=dtype))
    return b.finalize()


def test_stepwise_fp64_state_and_result(cuda_device):
    model = _column(torch.float64)
    crit = ag.ConvergenceCriteria(max_steps=3000, rtol=1e-7)
    opt = ag.PNCG(crit)
    fwd = ag.Forward(model, opt)
    problem, state = fwd.problem, fwd.state
    dm = model.dof_map
    g0 = problem.grad(state)
    d0 = problem.hess_diag(state).abs()
    mean0 = float(d0[d0 > 0].mean())

    opt_state = opt.init(problem, state, fwd.free)
    assert opt_state.n_steps == 0 and not opt_state.done and opt_state.beta == 0.0
    assert opt_state.direction.shape == g0.shape and not bool(opt_state.direction.any())
    assert opt_state.hess_damping_state.factor == 0.0
    assert math.isclose(opt_state.hess_damping_state.hess_diag_mean, mean0, rel_tol=1e-9)
    assert math.isclose(opt_state.convergence_state.grad_norm, float(g0.norm()), rel_tol=1e-9)

    done, result, steps = False, None, 0
    while not done:
        u_prev = dm.to_free(state.u)
        new_state, new_opt = opt.step(problem, state, opt_state)
        steps += 1
        ls = new_opt.line_search_state
        assert new_opt.n_steps == steps
        assert ls.f0 == opt_state.line_search_state.f_alpha
        if ls.ok:  # Armijo: the energy does not rise
            assert ls.f_alpha <= ls.f0 + 1e-12 * abs(ls.f0)
        # the step taken is alpha * direction (the logged step_direction)
        step = dm.to_free(new_state.u) - u_prev
        expect = ls.alpha * new_opt.direction
        scale = 1.0 + float(new_state.u.abs().max())
        assert float((step - expect).abs().max()) <= 1e-12 * scale, steps
        if steps == 1:  # beta = 0 and g0 = -f: p = -g0 / |diag0|
            pinv = torch.where(d0 > 0, 1.0 / d0, torch.full_like(d0, 1.0 / mean0))
            torch.testing.assert_close(new_opt.direction, -pinv * g0, rtol=1e-9,
                                       atol=1e-12 * float((pinv * g0).abs().max()))
        assert new_opt.hess_damping_state.hess_diag_mean > 0.0
        state, opt_state = new_state, new_opt
        done, result = opt.terminate(problem, state, opt_state)
        assert steps <= crit.max_steps
    assert result == ag.Result.PRIMARY_SUCCESS, result
    sol = opt.postprocess(problem, state, opt_state, result)
    assert sol.n_steps == steps and sol.relative_grad_norm <= 1e-7
    # the mean at the solution matches the diagonal evaluated there
    d = problem.hess_diag(state).abs()
    assert math.isclose(sol.hess_diag_mean, float(d[d > 0].mean()), rel_tol=1e-9)

    # the one-call solve takes the same iterations to the same point
    ref = ag.Forward(_column(torch.float64), ag.PNCG(crit))
    sol_ref = ref.step()
    assert sol_ref.n_steps == steps
    torch.testing.assert_close(ref.state.u, state.u, rtol=0, atol=1e-10)


def test_stepwise_fp32_direction(cuda_device):
    """FP32 (with the reference-state correction): the first direction is
    f / |diag| to FP32 accuracy, and steps move by alpha * direction."""
    model = _column(torch.float32)
    opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=50, rtol=1e-7))
    fwd = ag.Forward(model, opt)
    problem, state = fwd.problem, fwd.state
    g0 = problem.grad(state)
    d0 = problem.hess_diag(state).abs()
    opt_state = opt.init(problem, state, fwd.free)
    assert not bool(opt_state.direction.any())
    for k in range(5):
        u_prev = model.dof_map.to_free(state.u)
        state, opt_state = opt.step(problem, state, opt_state)
        if k == 0:
            torch.testing.assert_close(opt_state.direction, -g0 / d0, rtol=1e-4,
                                       atol=1e-6 * float((g0 / d0).abs().max()))
        step = model.dof_map.to_free(state.u) - u_prev
        expect = opt_state.line_search_state.alpha * opt_state.direction
        assert float((step - expect).abs().max()) <= 1e-5 * (1.0 + float(expect.abs().max())), k
