"""The oracle against golden vectors of the reference's own element kernels.

``tests/golden/reference_elements.npz`` was produced by
``tests/golden/make_elem_golden.py``, which runs the reference's unmodified
``warp/fem/_base.py`` kernels, its stable Neo-Hookean, muscle and ARAP
materials (``warp/fem/_stable_neo_hookean.py:17-103``,
``_stable_neo_hookean_muscle.py:18-114``, ``_arap.py:17-76``), the element
functions of ``warp/fem/func/*.py`` and ``warp/math/*.py``, and the region
precompute ``jax/fem/region/_region.py:84-108`` on NumPy in FP64.  These CPU
tests pin the FP64 oracle (and the C restatement) to them; the CUDA kernels
are checked against the same vectors in ``test_gpu_golden.py``.
"""

import pathlib

import numpy as np
import pytest

from oracle import fem_oracle as O

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "reference_elements.npz"
MESHES = ("tets", "grid")
MATERIALS = {"snh": O.Material.STABLE_NEO_HOOKEAN, "muscle": O.Material.STABLE_NEO_HOOKEAN_MUSCLE,
             "arap": O.Material.ARAP}
RTOL = 1e-12


@pytest.fixture(scope="module")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def case(g, mesh, mat):
    key = f"{mesh}__{mat}__"
    return g[f"{mesh}__points"], g[f"{mesh}__cells"], {k[len(key):]: v for k, v in g.items() if k.startswith(key)}


def oracle_potential(points, cells, c, mat):
    lam = c["lambda"] if mat != "arap" else None
    act = c["activation"] if mat == "muscle" else None
    return O.FemPotential.from_mesh(MATERIALS[mat], points, cells, mu=c["mu"], lam=lam, activation=act)


def test_golden_file_is_complete(golden):
    for mesh in MESHES:
        for mat in MATERIALS:
            _, cells, c = case(golden, mesh, mat)
            for k in ("u", "p", "mu", "dhdX", "dV", "F", "psi", "pk1", "fun", "grad", "hess_diag", "hess_prod",
                      "hess_quad"):
                assert k in c, (mesh, mat, k)
            assert c["dhdX"].shape == (cells.shape[0], 4, 3)
            # non-inverted deformations: the SVD convention does not enter
            assert np.linalg.det(c["F"]).min() > 0.0
            assert np.abs(c["fun"]).max() > 0.0 and np.abs(c["hess_quad"]).max() > 0.0


@pytest.mark.parametrize("mesh", MESHES)
def test_region_precompute_matches_reference(golden, mesh):
    points, cells, c = case(golden, mesh, "snh")
    dhdX, dV = O.region_compute_grad(points, cells)
    assert rel(dhdX, c["dhdX"]) < RTOL
    assert rel(dV, c["dV"]) < RTOL


@pytest.mark.parametrize("mat", list(MATERIALS))
@pytest.mark.parametrize("mesh", MESHES)
def test_oracle_elements_match_reference(golden, mesh, mat):
    points, cells, c = case(golden, mesh, mat)
    pot = oracle_potential(points, cells, c, mat)
    u, p = c["u"], c["p"]
    assert rel(pot._F(u), c["F"]) < RTOL
    assert rel(pot.energy_density(u), c["psi"]) < RTOL
    assert rel(pot.pk1(u), c["pk1"]) < RTOL
    assert rel(pot.fun(u), c["fun"][0]) < RTOL
    assert rel(pot.grad(u), c["grad"]) < RTOL
    assert rel(pot.hess_diag(u), c["hess_diag"]) < RTOL
    assert rel(pot.hess_quad(u, p), c["hess_quad"][0]) < RTOL
    if mat == "arap":
        # the reference's kernel as written (operands of h4_prod / h5_prod
        # swapped, _arap.py:55-56) and as intended (declared order)
        F = pot._F(u)
        as_called = O.arap_hess_prod_as_called(F, p[cells], pot.dhdX, pot.mu) * pot.dV[:, None, None]
        assert rel(pot._scatter(u.shape[0], as_called), c["hess_prod"]) < RTOL
        assert rel(pot.hess_prod(u, p), c["arap_hess_prod_intended"]) < RTOL
        assert rel(c["hess_prod"], c["arap_hess_prod_intended"]) > 1e-3  # the two differ
    else:
        assert rel(pot.hess_prod(u, p), c["hess_prod"]) < RTOL


@pytest.mark.parametrize("mat", ["snh", "arap"])
@pytest.mark.parametrize("mesh", MESHES)
def test_c_restatement_matches_reference(golden, mesh, mat):
    build_c = pytest.importorskip("oracle.build_c")
    try:
        build_c.load()
    except RuntimeError as e:  # no compiler
        pytest.skip(str(e))
    points, cells, c = case(golden, mesh, mat)
    pot = oracle_potential(points, cells, c, mat)
    cm = build_c.CModel(int(MATERIALS[mat]), pot.cells, pot.dhdX, pot.dV, pot.mu, pot.lam, points.shape[0])
    r = cm.eval(c["u"], c["p"])
    tol = 1e-10
    assert rel(r["fun"], c["fun"][0]) < tol
    assert rel(r["grad"], c["grad"]) < tol
    assert rel(r["hess_diag"], c["hess_diag"]) < tol
    assert rel(r["hess_quad"], c["hess_quad"][0]) < tol
    assert rel(r["hess_prod"], c["arap_hess_prod_intended"] if mat == "arap" else c["hess_prod"]) < tol
