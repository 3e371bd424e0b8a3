"""Mesh attribute access and the region precompute.

``Region`` mirrors ``liblaf.apple.jax.fem.Region`` (jax/fem/region/_region.py):
``from_pyvista(mesh, grad=True)`` computes, per tetrahedron with the 1-point
rule (quadrature/_tetra.py:14-15), the shape-function gradients ``dhdX``
(c, q=1, a=4, J=3) and ``dV`` (c, q=1) = det(Dm)/6.  The arithmetic runs in
the native library (``agb_region_compute``).  Attribute names follow
common/attr_name.py:4-44.
"""

from __future__ import annotations

import ctypes
import logging

import numpy as np

from . import _lib

logger = logging.getLogger(__name__)

# common/attr_name.py: AttrName.vtk
MU = "mu"
LAMBDA = "lambda"
FRACTION = "Fraction"
FIXED_MASK = "FixedMask"
FIXED_VALUE = "FixedValue"
GLOBAL_POINT_ID = "GlobalPointId"
FORCE = "Force"
ACTIVATION = "Activation"

TETRA = 10  # VTK_TETRA


def mesh_points(mesh) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(mesh.points, dtype=np.float64).reshape(-1, 3))


def mesh_cells(mesh) -> np.ndarray:
    """(n_cells, 4) local point ids of a TetMesh or a pyvista UnstructuredGrid."""
    cells = getattr(mesh, "cells_dict", None)
    if isinstance(cells, dict) and TETRA in cells:
        c = cells[TETRA]
    else:
        c = mesh.cells
    c = np.asarray(c)
    if c.ndim == 1:  # pyvista flat [4, i, j, k, l, ...]
        c = c.reshape(-1, 5)[:, 1:]
    return np.ascontiguousarray(c.astype(np.int32).reshape(-1, 4))


def point_data(mesh) -> dict:
    return mesh.point_data


def cell_data(mesh) -> dict:
    return mesh.cell_data


def cells_global(mesh) -> np.ndarray:
    """Local cells mapped through GlobalPointId (geometry/_geometry.py:39-49);
    the identity when the mesh carries none."""
    c = mesh_cells(mesh)
    pd = point_data(mesh)
    if GLOBAL_POINT_ID in pd:
        gid = np.asarray(pd[GLOBAL_POINT_ID]).astype(np.int32)
        c = gid[c]
    return np.ascontiguousarray(c.astype(np.int32))


def region_compute(points: np.ndarray, cells: np.ndarray, fraction: np.ndarray | None = None):
    """(dhdX (c, 4, 3), dV (c,)) in FP64 via the native library."""
    points = np.ascontiguousarray(points, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int32)
    n = cells.shape[0]
    dhdX = np.empty((n, 4, 3), np.float64)
    dV = np.empty((n,), np.float64)
    frac = None if fraction is None else np.ascontiguousarray(fraction, dtype=np.float64)
    bad = ctypes.c_int32(0)
    _lib.call(
        "agb_region_compute",
        n,
        cells.ctypes.data,
        points.shape[0],
        points.ctypes.data,
        None if frac is None else frac.ctypes.data,
        dhdX.ctypes.data,
        dV.ctypes.data,
        ctypes.byref(bad),
    )
    if bad.value:
        logger.warning("dV <= 0")  # jax/fem/region/_region.py:98-99
    return dhdX, dV


class Region:
    """Tetrahedral region with its FEM precompute."""

    def __init__(self, mesh, *, grad: bool = False):
        self.mesh = mesh
        self.points = mesh_points(mesh)
        self.cells_local = mesh_cells(mesh)
        self.cells_global = cells_global(mesh)
        self.dhdX = None
        self.dV = None
        if grad:
            self.compute_grad()

    @classmethod
    def from_pyvista(cls, mesh, *, grad: bool = False) -> "Region":
        return cls(mesh, grad=grad)

    from_mesh = from_pyvista

    @property
    def n_cells(self) -> int:
        return int(self.cells_local.shape[0])

    @property
    def cell_data(self) -> dict:
        return cell_data(self.mesh)

    @property
    def point_data(self) -> dict:
        return point_data(self.mesh)

    def compute_grad(self) -> None:
        dhdX, dV = region_compute(self.points, self.cells_local)
        self.dhdX = dhdX[:, None]  # (c, q=1, a, J)
        self.dV = dV[:, None]  # (c, q=1)
