"""Seeded synthetic tetrahedral meshes for the benchmark configurations.

The reference builds its meshes with tetwild from surfaces
(``benches/test_aggregation.py:23-27``) and its experiment meshes are Git-LFS
pointers, so every configuration here is generated: a structured grid split
into 5 tets per cube with alternating parity (faces conform across cubes),
and an irregular Delaunay ball.  Lame parameters follow
``common/_moduli.py:5-10``.
"""

from __future__ import annotations

import dataclasses

import numpy as np

# 5-tet split of a unit cube.  Corners are indexed by bits (x, y, z).  The
# "even" split keeps the regular tetrahedron on corners {000,110,101,011};
# the "odd" split mirrors it so that shared face diagonals match.
_EVEN = (
    (0b100, 0b000, 0b110, 0b101),  # corner tet at 100
    (0b010, 0b000, 0b011, 0b110),  # corner tet at 010
    (0b001, 0b000, 0b101, 0b011),  # corner tet at 001
    (0b111, 0b110, 0b011, 0b101),  # corner tet at 111
    (0b000, 0b110, 0b011, 0b101),  # central tet
)


def _mirror(c: int) -> int:
    return c ^ 0b001  # flip z: swaps the two corner groups


_ODD = tuple(tuple(_mirror(c) for c in t) for t in _EVEN)


@dataclasses.dataclass
class TetMesh:
    """Minimal mesh container with the attribute names the reference reads
    from pyvista (``points``, ``cells``, ``point_data``, ``cell_data``)."""

    points: np.ndarray  # (N_v, 3) float64 rest positions
    cells: np.ndarray  # (N_t, 4) int32
    point_data: dict = dataclasses.field(default_factory=dict)
    cell_data: dict = dataclasses.field(default_factory=dict)

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_cells(self) -> int:
        return int(self.cells.shape[0])

    def volume(self) -> float:
        p = self.points[self.cells]
        D = np.stack([p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]], axis=-1)
        return float(np.abs(np.linalg.det(D)).sum() / 6.0)


def _orient(points: np.ndarray, cells: np.ndarray) -> np.ndarray:
    p = points[cells]
    D = np.stack([p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]], axis=-1)
    neg = np.linalg.det(D) < 0
    cells = cells.copy()
    cells[neg, 2], cells[neg, 3] = cells[neg, 3].copy(), cells[neg, 2].copy()
    return cells


def grid(nx: int, ny: int, nz: int, h: float = None, lengths=None) -> TetMesh:
    """(nx+1)(ny+1)(nz+1) vertices, 5 nx ny nz tets; x varies fastest."""
    if lengths is None:
        h = 1.0 / nx if h is None else h
        lengths = (nx * h, ny * h, nz * h)
    xs = np.linspace(0.0, lengths[0], nx + 1)
    ys = np.linspace(0.0, lengths[1], ny + 1)
    zs = np.linspace(0.0, lengths[2], nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    points = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=-1)

    def vid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    parity = (i + j + k) & 1
    cells = np.empty((i.size, 5, 4), dtype=np.int64)
    for split, sel in ((_EVEN, parity == 0), (_ODD, parity == 1)):
        for t, tet in enumerate(split):
            for a, c in enumerate(tet):
                dx, dy, dz = (c >> 2) & 1, (c >> 1) & 1, c & 1
                cells[sel, t, a] = vid(i[sel] + dx, j[sel] + dy, k[sel] + dz)
    cells = cells.reshape(-1, 4)
    cells = _orient(points, cells)
    return TetMesh(points=points, cells=cells.astype(np.int32))


def ball(n_interior: int, n_shell: int, seed: int = 0, min_quality: float = 0.05) -> TetMesh:
    """Delaunay tetrahedralisation of points uniform in the unit ball plus a
    shell on the unit sphere; vertex order is a seeded random permutation;
    inverted tets are re-oriented and slivers dropped: quality
    q = 12 (3V)^(2/3) / sum of squared edge lengths (1 for a regular tet)
    below ``min_quality`` (about 0.2% of the tets at 0.05)."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n_interior, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rng.random(n_interior) ** (1.0 / 3.0)
    interior = d * r[:, None]
    s = rng.normal(size=(n_shell, 3))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    pts = np.concatenate([interior, s], axis=0)
    perm = rng.permutation(pts.shape[0])
    pts = pts[perm]
    tri = Delaunay(pts)
    cells = tri.simplices.astype(np.int64)
    cells = _orient(pts, cells)
    p = pts[cells]
    D = np.stack([p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]], axis=-1)
    vol = np.linalg.det(D) / 6.0
    edges = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))
    l2 = sum(((p[:, a] - p[:, b]) ** 2).sum(-1) for a, b in edges)
    q = 12.0 * np.cbrt(3.0 * np.abs(vol)) ** 2 / l2
    keep = (vol > 0) & (q >= min_quality)
    cells = cells[keep]
    used = np.zeros(pts.shape[0], bool)
    used[cells.ravel()] = True
    remap = np.cumsum(used) - 1
    return TetMesh(points=pts[used], cells=remap[cells].astype(np.int32))


def lame_converter(E, nu):
    """(lambda, mu) from Young's modulus and Poisson ratio (``common/_moduli.py:5-10``)."""
    E = np.asarray(E, dtype=np.float64)
    nu = np.asarray(nu, dtype=np.float64)
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    return lam, mu


def face_mask(mesh: TetMesh, axis: int, side: str, tol: float = 1e-9) -> np.ndarray:
    x = mesh.points[:, axis]
    v = x.min() if side == "min" else x.max()
    return np.abs(x - v) <= tol * max(1.0, abs(v))


def lumped_gravity(mesh: TetMesh, rho: float, g=(0.0, 0.0, -9.8)) -> np.ndarray:
    """Per-vertex force rho g sum_e V_e / 4 (lumped mass)."""
    p = mesh.points[mesh.cells]
    D = np.stack([p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]], axis=-1)
    vol = np.abs(np.linalg.det(D)) / 6.0
    m = np.zeros(mesh.n_points)
    np.add.at(m, mesh.cells.ravel(), np.repeat(vol / 4.0, 4))
    return rho * m[:, None] * np.asarray(g, np.float64)[None, :]


def batch_case(k: int, rng: np.random.Generator, dims=(4, 40), h: float = 0.05):
    """One mesh of the batched workload: a grid with (nx, ny, nz) ~ U{dims}
    cells per axis, stable Neo-Hookean with E ~ U[1e3, 1e5], nu ~ U[0.3, 0.49],
    density 1000, one random Dirichlet face (all three components fixed) and
    a random gravity direction.  Returns (mesh with FixedMask / FixedValue and
    mu / lambda cell data, per-vertex force)."""
    nx, ny, nz = (int(v) for v in rng.integers(dims[0], dims[1] + 1, size=3))
    m = grid(nx, ny, nz, h=h)
    E = float(rng.uniform(1e3, 1e5))
    nu = float(rng.uniform(0.3, 0.49))
    lam, mu = lame_converter(E, nu)
    m.cell_data["mu"] = np.full(m.n_cells, mu)
    m.cell_data["lambda"] = np.full(m.n_cells, lam)
    face = int(rng.integers(0, 6))
    mask = np.zeros((m.n_points, 3), bool)
    mask[face_mask(m, face // 2, "min" if face % 2 == 0 else "max")] = True
    m.point_data["FixedMask"] = mask
    m.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    g = rng.normal(size=3)
    g *= 9.8 / np.linalg.norm(g)
    return m, lumped_gravity(m, 1000.0, g)
