"""The FP32 vertex pass streams a chunk of 256 vertices' inputs into shared
memory with bulk copies, with at most 768 of the chunk's slots; a chunk with
more slots reads the rest from global memory.  With tiles of 8 elements,
every vertex lies in about five tiles, so nearly every chunk has more than
768 slots and the solve goes through that path.  The same solve with the
default tiles (no chunk overflows) and the FP64 C restatement's solve must
agree with it: 1e-4 of the bounding-box diagonal, the FP32 bar.  (A cube of
E = 1e6 sagging under gravity: strains of about 1e-2, one equilibrium.)"""

import ctypes

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import _lib, meshgen
from oracle import build_c
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def _problem():
    m = meshgen.grid(8, 8, 8)
    lam, mu = meshgen.lame_converter(1e6, 0.45)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    return m, mu, lam, mask, meshgen.lumped_gravity(m, 1000.0)


def _solve(m, mu, lam, mask, f, tile_elems):
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    b = ag.ModelBuilder(dtype=torch.float32)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, tile_elems=tile_elems))
    fm = meshgen.TetMesh(m.points, m.cells)
    fm.point_data["Force"] = f
    fm.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fm))
    fwd = ag.Forward(b.finalize(), ag.PNCG(ag.ConvergenceCriteria(max_steps=20000, rtol=1e-6)))
    sol = fwd.step()
    assert sol.result == ag.Result.PRIMARY_SUCCESS, sol
    return fwd.state.u.double().cpu().numpy()


def test_overflowing_chunks_match_default_tiles_and_oracle(cuda_device):
    m, mu, lam, mask, f = _problem()
    # the plan with 8-element tiles: slots per vertex = tiles that hold it
    tile = np.empty(m.n_cells, np.int32)
    nt, ng = ctypes.c_int32(), ctypes.c_int32()
    cells = np.ascontiguousarray(m.cells, np.int32)
    pts = np.ascontiguousarray(m.points, np.float64)
    _lib.call("agb_plan_tiles", m.n_points, m.n_cells, cells.ctypes.data, pts.ctypes.data, 8, ctypes.byref(nt),
              ctypes.byref(ng), tile.ctypes.data, None, None)
    pairs = np.unique(np.stack([np.repeat(tile, 4), cells.reshape(-1)], 1), axis=0)
    assert len(pairs) / m.n_points > 768 / 256 + 1  # an average chunk overflows its 768 staged slots
    u_small = _solve(m, mu, lam, mask, f, 8)
    u_default = _solve(m, mu, lam, mask, f, 0)
    dhdX, dV = O.region_compute_grad(m.points, m.cells)
    cm = build_c.CModel(1, m.cells, dhdX, dV, np.full(m.n_cells, mu), np.full(m.n_cells, lam), m.n_points,
                        mask=mask, force=f)
    u_ref, _ = cm.pncg(np.zeros((m.n_points, 3)), max_steps=50000, rtol=1e-10)
    diag = float(np.linalg.norm(m.points.max(0) - m.points.min(0)))
    assert np.abs(u_small - u_default).max() < 1e-4 * diag
    assert np.abs(u_small - u_ref).max() < 1e-4 * diag
