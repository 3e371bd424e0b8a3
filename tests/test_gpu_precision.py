"""FP32 solves below the FP32 force-rounding floor (GB300).

Without the reference-state correction the FP32 gradient of a gravity-loaded
column is dominated by the rounding of element forces much larger than the
residual, and PNCG stalls near ||g||/||g0|| ~ 1e-5.  With it (FP32 stable
Neo-Hookean solvers), the element pass evaluates f_e(x) - f_e(x_ref) and
g(x_ref) is refreshed in FP64, so FP32 reaches 1e-7 here, and the answer
(rounded to FP32 on output) matches the FP64 oracle to 1e-6 of the
bounding-box diagonal.  The true gradient at that FP32-rounded answer is only
as small as the rounding of u allows (~1e-5 relative here), which is why the
solve keeps positions as float-float pairs internally."""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def test_fp32_gravity_column_reaches_1e7(cuda_device):
    m = meshgen.grid(6, 5, 8)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    f = meshgen.lumped_gravity(m, 1000.0)
    b = ag.ModelBuilder()
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh))
    fm = meshgen.TetMesh(m.points, m.cells)
    fm.point_data["Force"] = f
    fm.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fm))
    fwd = ag.Forward(b.finalize(), ag.PNCG(ag.ConvergenceCriteria(max_steps=20000, rtol=1e-7)))
    sol = fwd.step()
    assert sol.result == ag.Result.PRIMARY_SUCCESS, sol
    ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=mu, lam=lam)
    om = O.Model(O.DofMap(m.n_points, mask, np.zeros((m.n_points, 3))), [ora],
                 O.ExternalForce(np.arange(m.n_points), f))
    u_ref, _ = O.solve_model(om, rtol=1e-11, max_steps=20000)
    diag = float(np.linalg.norm(m.points.max(0) - m.points.min(0)))
    u = fwd.state.u.double().cpu().numpy()
    assert float(np.abs(u - u_ref).max()) < 1e-6 * diag
