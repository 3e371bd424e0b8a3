"""Failure handling and checkpoint / resume of the device PNCG (GB300).

Failures are injected on the host, never by faulting the GPU: a NaN in the
initial displacement, an exhausted step budget, a model whose free DOFs have
no stiffness at all, a checkpoint loaded into the wrong solver.  A checkpoint
taken mid-solve and restored continues bit for bit."""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from apple_gb300.forward import ModelState

pytestmark = pytest.mark.gpu


def _column(n=(4, 4, 6), dtype=torch.float32, extra_points=0, fix_all_mesh=False, fixed_face=("z", "min"), E=1e4):
    m = meshgen.grid(*n)
    pts = m.points
    if extra_points:
        pts = np.concatenate([pts, 5.0 + np.arange(3 * extra_points, dtype=float).reshape(-1, 3)])
    n_pts = pts.shape[0]
    lam, mu = meshgen.lame_converter(E, 0.45)
    mesh = ag.with_lame(meshgen.TetMesh(pts, m.cells), mu, lam)
    mask = np.zeros((n_pts, 3), bool)
    if fix_all_mesh:
        mask[: m.n_points] = True
    else:
        mask[: m.n_points][meshgen.face_mask(m, "xyz".index(fixed_face[0]), fixed_face[1])] = True
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((n_pts, 3))
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, dtype=dtype))
    f = np.zeros((n_pts, 3))
    f[: m.n_points] = meshgen.lumped_gravity(m, 1000.0)
    fm = meshgen.TetMesh(pts, m.cells)
    fm.point_data["Force"] = f
    fm.point_data["GlobalPointId"] = np.arange(n_pts)
    b.add_potential(ag.ExternalForce.from_pyvista(fm, dtype=dtype))
    return b.finalize()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_checkpoint_resume_is_exact(dtype, cuda_device):
    model = _column(dtype=dtype)
    opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=10_000, rtol=1e-7))
    fwd = ag.Forward(model, opt)
    sv = opt.solver(fwd.problem)
    sv.reset(fwd.state.u)
    sv.iterate(15)
    blob = sv.save_state()
    sv.iterate(25)
    u_a = torch.empty_like(fwd.state.u)
    st_a = sv.read(u_a)
    sv.load_state(blob)
    sv.iterate(25)
    u_b = torch.empty_like(fwd.state.u)
    st_b = sv.read(u_b)
    assert st_a.n_steps == st_b.n_steps == 40
    assert torch.equal(u_a, u_b)
    assert st_a.grad_norm == st_b.grad_norm
    # an identically built solver resumes the same way
    opt2 = ag.PNCG(ag.ConvergenceCriteria(max_steps=10_000, rtol=1e-7))
    sv2 = opt2.solver(ag.ForwardProblem(model))
    sv2.load_state(blob)
    sv2.iterate(25)
    u_c = torch.empty_like(fwd.state.u)
    sv2.read(u_c)
    assert torch.equal(u_a, u_c)


def test_checkpoint_rejected_by_another_solver(cuda_device):
    a, b = _column(n=(4, 4, 6)), _column(n=(4, 4, 7))
    opt_a, opt_b = ag.PNCG(), ag.PNCG()
    sa = opt_a.solver(ag.ForwardProblem(a))
    sa.reset(ag.Forward(a, opt_a).state.u)
    sb = opt_b.solver(ag.ForwardProblem(b))
    with pytest.raises(RuntimeError):
        sb.load_state(sa.save_state())
    bad = sa.save_state()
    bad[:8] = 0  # not a checkpoint
    with pytest.raises(RuntimeError):
        sa.load_state(bad)
    good = sa.save_state()
    with pytest.raises(RuntimeError, match="bytes"):
        sa.load_state(good[:-1])  # truncated
    with pytest.raises(RuntimeError, match="bytes"):
        sa.load_state(torch.cat([good, torch.zeros(8, dtype=torch.uint8)]))  # trailing data
    sa.load_state(good)  # the intact blob still loads


def test_checkpoint_rejected_by_a_model_of_the_same_size(cuda_device):
    """Same vertex count, precision and correction setting, but another fixed
    face, another material or other solver parameters: the fingerprint in the
    header refuses the checkpoint."""
    base = _column(n=(4, 4, 6))
    opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=1000, rtol=1e-7))
    sa = opt.solver(ag.ForwardProblem(base))
    sa.reset(ag.Forward(base, opt).state.u)
    sa.iterate(5)
    blob = sa.save_state()
    other_face = _column(n=(4, 4, 6), fixed_face=("z", "max"))
    stiffer = _column(n=(4, 4, 6), E=2e4)
    for model, crit in ((other_face, dict(rtol=1e-7)), (stiffer, dict(rtol=1e-7)), (base, dict(rtol=1e-8))):
        o = ag.PNCG(ag.ConvergenceCriteria(max_steps=1000, **crit))
        sv = o.solver(ag.ForwardProblem(model))
        with pytest.raises(RuntimeError, match="another model"):
            sv.load_state(blob)
    # an identically built model and solver accept it
    o = ag.PNCG(ag.ConvergenceCriteria(max_steps=1000, rtol=1e-7))
    o.solver(ag.ForwardProblem(_column(n=(4, 4, 6)))).load_state(blob)


def test_nan_input_ends_with_nan_encountered(cuda_device):
    model = _column()
    fwd = ag.Forward(model, ag.PNCG(ag.ConvergenceCriteria(max_steps=100, rtol=1e-6)))
    u = fwd.state.u.clone()
    free = np.flatnonzero(~model.dof_map.fixed_mask.reshape(-1))
    u.view(-1)[int(free[-1])] = float("nan")  # a free DOF: the solve starts from it
    fwd.state = ModelState(u=u)
    sol = fwd.step()
    assert sol.result == ag.Result.NAN_ENCOUNTERED, sol


def test_step_budget_exhaustion(cuda_device):
    model = _column()
    sol = ag.Forward(model, ag.PNCG(ag.ConvergenceCriteria(max_steps=3, rtol=1e-12))).step()
    assert sol.result == ag.Result.MAX_STEPS_REACHED and sol.n_steps == 3, sol


def test_free_dofs_without_stiffness(cuda_device):
    """Every mesh vertex fixed; the only free DOFs belong to points no cell
    references: zero gradient and zero diagonal (the preconditioner's mean
    fallback), so the solve ends at once and moves nothing."""
    model = _column(extra_points=2, fix_all_mesh=True)
    fwd = ag.Forward(model, ag.PNCG(ag.ConvergenceCriteria(max_steps=100, rtol=1e-6)))
    u0 = fwd.state.u.clone()
    sol = fwd.step()
    assert sol.result == ag.Result.PRIMARY_SUCCESS, sol
    assert torch.equal(fwd.state.u, u0)


def test_solver_rejects_a_model_without_cells(cuda_device):
    """A model whose only FEM potential has no cells has nothing to iterate:
    the solver is refused at creation with a status, not at the first launch."""
    m = meshgen.grid(2, 2, 2)
    empty = ag.with_lame(meshgen.TetMesh(m.points, np.zeros((0, 4), np.int32)), 1.0e3, 1.0e4)
    b = ag.ModelBuilder()
    b.add_vertices(meshgen.TetMesh(m.points, m.cells))
    b.add_potential(ag.StableNeoHookean.from_pyvista(empty))
    model = b.finalize()
    with pytest.raises(RuntimeError, match="no cells"):
        ag.PNCG().solver(ag.ForwardProblem(model))
