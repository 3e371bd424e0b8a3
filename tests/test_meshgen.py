"""The synthetic meshes behind every workload: the 5-tet grid is conforming
(every interior face shared by exactly two tets, the boundary faces by one),
positively oriented and fills its box; the Delaunay ball is positively
oriented with its slivers dropped; the batched cases are reproducible."""

import collections

import numpy as np

from apple_gb300 import meshgen


def _faces(cells):
    c = np.asarray(cells)
    f = np.concatenate([c[:, [1, 2, 3]], c[:, [0, 2, 3]], c[:, [0, 1, 3]], c[:, [0, 1, 2]]])
    return collections.Counter(map(tuple, np.sort(f, axis=1)))


def _volumes(m):
    p = m.points[m.cells]
    return np.linalg.det(np.stack([p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]], axis=-1)) / 6.0


def test_grid_is_conforming_and_fills_its_box():
    nx, ny, nz = 4, 3, 5
    m = meshgen.grid(nx, ny, nz, h=0.5)
    assert m.n_cells == 5 * nx * ny * nz and m.n_points == (nx + 1) * (ny + 1) * (nz + 1)
    v = _volumes(m)
    assert np.all(v > 0)
    assert abs(v.sum() - nx * ny * nz * 0.125) < 1e-12
    counts = collections.Counter(_faces(m.cells).values())
    assert set(counts) == {1, 2}
    boundary = 2 * 2 * (nx * ny + ny * nz + nx * nz)  # two triangles per boundary square
    assert counts[1] == boundary


def test_ball_is_oriented_and_has_no_slivers():
    m = meshgen.ball(2000, 400, seed=5)
    v = _volumes(m)
    assert np.all(v > 0)
    assert set(_faces(m.cells).values()) <= {1, 2}
    r = np.linalg.norm(m.points, axis=1)
    assert r.max() <= 1.0 + 1e-12


def test_batch_cases_are_reproducible():
    a = [meshgen.batch_case(k, np.random.default_rng(7), dims=(2, 5)) for k in range(3)]
    b = [meshgen.batch_case(k, np.random.default_rng(7), dims=(2, 5)) for k in range(3)]
    for (ma, fa), (mb, fb) in zip(a, b):
        np.testing.assert_array_equal(ma.cells, mb.cells)
        np.testing.assert_array_equal(fa, fb)
        np.testing.assert_array_equal(ma.point_data["FixedMask"], mb.point_data["FixedMask"])
        assert ma.point_data["FixedMask"].any()
        assert np.isclose(np.linalg.norm(fa.sum(0)) / (1000.0 * 9.8), ma.volume(), rtol=1e-9)
