"""The 64x64x96 grid and the irregular Delaunay ball at their full sizes (GB300).

* 64x64x96 cells (1,966,080 tets): FP32 energy, gradient and Hessian diagonal
  of the API path at a displaced state (30% stretch plus a smooth
  perturbation) against the FP64 C restatement of the reference kernels,
  stable Neo-Hookean (E = 1e5, nu = 0.49) and ARAP (mu = 1); bar 1e-5
  relative (L2 for vectors).
* The Delaunay ball (300,000 interior + 20,000 shell points, random vertex
  order, per-tet mu log-uniform in [1e3, 1e6], lambda = 10 mu): the tile /
  warp-group plan built twice is identical, keeps every cell's corner set and
  holds the per-slot distinctness the atomic-free scatter relies on; and the
  FP32 evaluation against the FP64 C restatement, as for the grid.
"""

import ctypes

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import _lib, meshgen
from oracle import build_c
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _compare(cls, material, m, mu, lam, u, cuda_device):
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.cell_data["mu"] = np.broadcast_to(mu, (m.n_cells,)).copy()
    if lam is not None:
        mesh.cell_data["lambda"] = np.broadcast_to(lam, (m.n_cells,)).copy()
    pot = cls.from_pyvista(mesh, dtype=torch.float32)
    U = torch.tensor(u, dtype=torch.float32, device=cuda_device)
    out = pot.eval(U, None, fun=True, grad=True, hess_diag=True)
    torch.cuda.synchronize(cuda_device)
    dhdX, dV = O.region_compute_grad(m.points, m.cells)
    cm = build_c.CModel(int(material), m.cells, dhdX, dV, mu, lam, m.n_points)
    ref = cm.eval(U.double().cpu().numpy(), None, flags=7)
    assert rel(out["fun"].item(), ref["fun"]) < TOL
    assert rel(out["grad"].cpu(), ref["grad"]) < TOL
    assert rel(out["hess_diag"].cpu(), ref["hess_diag"]) < TOL


@pytest.fixture(scope="module")
def grid64():
    m = meshgen.grid(64, 64, 96, h=1.0 / 64)
    assert m.n_cells == 1_966_080 and m.n_points == 409_825
    rng = np.random.default_rng(3)
    X = m.points - m.points.mean(0)
    u = np.zeros_like(m.points)
    u[:, 2] = 0.3 * (m.points[:, 2] - m.points[:, 2].min())
    u += 0.01 * np.sin(X @ rng.normal(size=(3, 3)) * 3.0)
    return m, u


@pytest.mark.parametrize("material", ["snh", "arap"])
def test_grid64_fp32_matches_fp64_restatement(grid64, material, cuda_device):
    m, u = grid64
    if material == "snh":
        lam, mu = meshgen.lame_converter(1e5, 0.49)
        _compare(ag.StableNeoHookean, O.Material.STABLE_NEO_HOOKEAN, m, mu, lam, u, cuda_device)
    else:
        _compare(ag.Arap, O.Material.ARAP, m, 1.0, None, u, cuda_device)


@pytest.fixture(scope="module")
def ball():
    m = meshgen.ball(300_000, 20_000, seed=0)
    assert 1_700_000 < m.n_cells < 2_200_000
    return m


def _plan(m):
    nc = m.n_cells
    cells = np.ascontiguousarray(m.cells, np.int32)
    pts = np.ascontiguousarray(m.points, np.float64)
    tile = np.empty(nc, np.int32)
    group = np.empty(nc, np.int32)
    slots = np.empty((nc, 4), np.int32)
    nt, ng = ctypes.c_int32(), ctypes.c_int32()
    _lib.call("agb_plan_tiles", m.n_points, nc, cells.ctypes.data, pts.ctypes.data, 0, ctypes.byref(nt),
              ctypes.byref(ng), tile.ctypes.data, group.ctypes.data, slots.ctypes.data)
    return nt.value, ng.value, tile, group, slots


def test_ball_plan_is_exact_and_reproducible(ball, cuda_device):
    a = _plan(ball)
    b = _plan(ball)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    nt, ng, tile, group, slots = a
    np.testing.assert_array_equal(np.sort(slots, axis=1), np.sort(ball.cells, axis=1))
    # per warp group and corner slot: distinct vertices
    for k in range(4):
        key = group.astype(np.int64) * ball.n_points + slots[:, k]
        assert np.unique(key).size == key.size, f"slot {k}"
    # tiles: at most 1024 elements; every group inside one tile
    assert np.all(np.bincount(tile, minlength=nt) <= 1024)
    tile_of_group = np.full(ng, -1, np.int64)
    tile_of_group[group] = tile
    assert np.all(tile_of_group[group] == tile)


def test_ball_fp32_matches_fp64_restatement(ball, cuda_device):
    rng = np.random.default_rng(4)
    mu = np.exp(rng.uniform(np.log(1e3), np.log(1e6), ball.n_cells))
    lam = 10.0 * mu
    u = 0.02 * np.sin(ball.points @ rng.normal(size=(3, 3)) * 2.0)
    _compare(ag.StableNeoHookean, O.Material.STABLE_NEO_HOOKEAN, ball, mu, lam, u, cuda_device)
