"""CUDA kernels against golden vectors of the reference's own element kernels
(GB300).

``tests/golden/reference_elements.npz`` holds what the reference's unmodified
``warp/fem/_base.py`` kernels compute for stable Neo-Hookean
(``_stable_neo_hookean.py:17-103``), the muscle
(``_stable_neo_hookean_muscle.py:18-114``) and ARAP (``_arap.py:17-76``) on
24 independent tets and a 2x2x2-cell grid: energy, gradient, clamped Hessian
diagonal, Hessian-vector product and clamped p^T H p (made by
``tests/golden/make_elem_golden.py``).  The five API methods run through the
C ABI in FP64 (bar 1e-9 relative) and FP32 (bar 1e-5 relative L2).  ARAP's
Hessian-vector product is compared with the reference's intended formula
(its h4_prod / h5_prod in their declared argument order).
"""

import pathlib

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "reference_elements.npz"
TOL = {torch.float64: 1e-9, torch.float32: 1e-5}
CLASSES = {"snh": ag.StableNeoHookean, "muscle": ag.StableNeoHookeanMuscle, "arap": ag.Arap}


@pytest.fixture(scope="module")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("mat", list(CLASSES))
@pytest.mark.parametrize("mesh_name", ["tets", "grid"])
def test_api_matches_reference_kernels(golden, mesh_name, mat, dtype, cuda_device):
    points, cells = golden[f"{mesh_name}__points"], golden[f"{mesh_name}__cells"]
    key = f"{mesh_name}__{mat}__"
    c = {k[len(key):]: v for k, v in golden.items() if k.startswith(key)}
    mesh = meshgen.TetMesh(points, cells)
    mesh.cell_data["mu"] = c["mu"]
    if mat != "arap":
        mesh.cell_data["lambda"] = c["lambda"]
    if mat == "muscle":
        mesh.cell_data["activation"] = c["activation"]
    pot = CLASSES[mat].from_pyvista(mesh, dtype=dtype)
    U = torch.tensor(c["u"], dtype=dtype, device=cuda_device)
    P = torch.tensor(c["p"], dtype=dtype, device=cuda_device)
    out = pot.eval(U, P, fun=True, grad=True, hess_diag=True, hess_prod=True, hess_quad=True)
    torch.cuda.synchronize(cuda_device)
    tol = TOL[dtype]
    assert rel(out["fun"].item(), c["fun"][0]) < tol
    assert rel(out["grad"].cpu(), c["grad"]) < tol
    assert rel(out["hess_diag"].cpu(), c["hess_diag"]) < tol
    assert rel(out["hess_quad"].item(), c["hess_quad"][0]) < tol
    hp = c["arap_hess_prod_intended"] if mat == "arap" else c["hess_prod"]
    assert rel(out["hess_prod"].cpu(), hp) < tol
