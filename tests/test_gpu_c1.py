"""The CPU-scale workload: a jittered unit cube of 10x10x10 cells (1,331
vertices, 5,000 tets), stable Neo-Hookean E = 1e4, nu = 0.45, gravity
(rho 1000), the z = 0 face fixed.  PNCG needs about a thousand iterations.

Checks, with the FP64 oracle evaluated at the GPU's answers: the FP32 solve
reaches ||g||/||g0|| <= 1e-6 and is an equilibrium of the FP64 model to 1e-4
(its output is rounded to FP32); the FP64 solve is one to 1e-7; both land in
the same equilibrium, whose energy the FP64 C restatement of the reference
loop reaches too (to 1e-9; it ends in a failed line search near 1e-6).  (The
gravity load is about E / L here: the cube sags by more than its height,
through inverted elements, which stable Neo-Hookean allows.)"""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from oracle import build_c
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def _c1():
    m = meshgen.grid(10, 10, 10)
    rng = np.random.default_rng(0)
    bottom = meshgen.face_mask(m, 2, "min")
    m.points[~bottom] += rng.uniform(-0.01, 0.01, size=(int((~bottom).sum()), 3)) * 0.1
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    mask = np.zeros((m.n_points, 3), bool)
    mask[bottom] = True
    f = meshgen.lumped_gravity(m, 1000.0)
    return m, mu, lam, mask, f


def _model(m, mu, lam, mask, f, dtype):
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    b = ag.ModelBuilder(dtype=dtype)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, dtype=dtype))
    fm = meshgen.TetMesh(m.points, m.cells)
    fm.point_data["Force"] = f
    fm.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fm, dtype=dtype))
    return b.finalize()


def test_c1_cube_fp32_and_fp64_against_the_oracle(cuda_device):
    m, mu, lam, mask, f = _c1()
    pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=mu, lam=lam)
    om = O.Model(O.DofMap(m.n_points, mask, np.zeros((m.n_points, 3))), [pot],
                 O.ExternalForce(np.arange(m.n_points), f))
    free = ~mask
    g0 = np.linalg.norm(om.grad(np.zeros((m.n_points, 3)))[free])

    def rel_grad(u):
        return np.linalg.norm(om.grad(u)[free]) / g0

    sols = {}
    for dtype, rtol, bound in ((torch.float32, 1e-6, 1e-4), (torch.float64, 1e-8, 1e-7)):
        fwd = ag.Forward(_model(m, mu, lam, mask, f, dtype),
                         ag.PNCG(ag.ConvergenceCriteria(max_steps=20000, rtol=rtol)))
        sol = fwd.step()
        # FP64 may end in a rejected line search once f(x + t p) - f(x) is below its resolution
        ok = (ag.Result.PRIMARY_SUCCESS,) if dtype == torch.float32 else (ag.Result.PRIMARY_SUCCESS,
                                                                          ag.Result.LINE_SEARCH_FAILED)
        assert sol.result in ok, (dtype, sol)
        u = fwd.state.u.double().cpu().numpy()
        assert rel_grad(u) < bound, (dtype, rel_grad(u))
        sols[dtype] = u
    # FP32 and FP64 end in the same equilibrium
    diag = np.linalg.norm(m.points.max(0) - m.points.min(0))
    assert np.abs(sols[torch.float32] - sols[torch.float64]).max() < 1e-3 * diag
    # ... as the C restatement of the reference loop (FP64): the same energy
    dhdX, dV = O.region_compute_grad(m.points, m.cells)
    cm = build_c.CModel(1, m.cells, dhdX, dV, np.full(m.n_cells, mu), np.full(m.n_cells, lam), m.n_points,
                        mask=mask, force=f)
    u_c, _ = cm.pncg(np.zeros((m.n_points, 3)), max_steps=20000, rtol=1e-10)
    e_gpu, e_c = om.fun(sols[torch.float64]), om.fun(u_c)
    assert abs(e_gpu - e_c) <= 1e-9 * abs(e_c)
