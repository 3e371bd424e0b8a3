"""The benchmark workloads on the host (no GPU): sizes and boundary
conditions of the headline grid and of the other configurations, as the
published configurations state them."""

import numpy as np
import pytest

import bench
from apple_gb300 import meshgen


def test_headline_grid_is_the_1_5m_tet_configuration():
    m, mu, lam, mask, fv = bench._mesh(False)
    assert (m.n_cells, m.n_points) == (1_500_000, 314_721)
    # E = 1e5, nu = 0.49
    assert mu == pytest.approx(1e5 / (2 * 1.49))
    assert lam == pytest.approx(1e5 * 0.49 / (1.49 * (1 - 0.98)))
    z = m.points[:, 2]
    bottom, top = np.isclose(z, z.min()), np.isclose(z, z.max())
    assert bottom.sum() == top.sum() == 51 * 51
    # z = 0 end fixed; z = max end displaced by +30% of the length along z
    assert mask[bottom].all() and mask[top].all() and not mask[~(bottom | top)].any()
    np.testing.assert_allclose(fv[top], np.tile([0.0, 0.0, 0.3 * z.max()], (top.sum(), 1)))
    assert not fv[~top].any()
    # positive volumes, and the cells tile the box exactly
    X = m.points[m.cells]
    vol = np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0])) / 6.0
    ext = m.points.max(0) - m.points.min(0)
    assert np.abs(vol).min() > 0
    assert np.abs(vol).sum() == pytest.approx(np.prod(ext), rel=1e-12)


@pytest.mark.parametrize("dims,n_cells,n_points", [
    ((64, 64, 96), 1_966_080, 409_825),  # the 64x64x96 grid
    ((24, 24, 48), 138_240, 30_625),     # the adjoint grid
    ((10, 10, 10), 5_000, 1_331),        # the CPU-scale cube
])
def test_grid_sizes(dims, n_cells, n_points):
    m = meshgen.grid(*dims, h=1.0 / dims[0])
    assert (m.n_cells, m.n_points) == (n_cells, n_points)
