"""The product's DOF map and its builder on the host (no GPU): global point
ids over several meshes (forward/dof_map/_builder.py:41-50), per-component
fixed masks and values (the same file, add_fixed), and the free / full
gather and scatter (forward/dof_map/_dof_map.py:30-49), checked against the
oracle's DofMap."""

import numpy as np
import torch

from apple_gb300 import meshgen
from apple_gb300.model import DofMapBuilder
from oracle import fem_oracle as O


def test_builder_over_two_meshes_matches_the_oracle():
    a, b = meshgen.grid(2, 2, 2), meshgen.grid(3, 2, 2)
    bld = DofMapBuilder()
    bld.add_vertices(a)
    bld.add_vertices(b)
    np.testing.assert_array_equal(a.point_data["GlobalPointId"], np.arange(a.n_points))
    np.testing.assert_array_equal(b.point_data["GlobalPointId"], a.n_points + np.arange(b.n_points))
    rng = np.random.default_rng(3)
    mask = rng.random((b.n_points, 3)) < 0.4
    vals = rng.normal(size=(b.n_points, 3))
    b.point_data["FixedMask"] = mask
    b.point_data["FixedValue"] = vals
    bld.add_fixed(b)
    dm = bld.finalize(dtype=torch.float64, device="cpu")
    n = a.n_points + b.n_points
    assert dm.n_points == n and dm.n_fixed == int(mask.sum()) and dm.n_free == 3 * n - int(mask.sum())

    full_mask = np.zeros((n, 3), bool)
    full_mask[a.n_points:] = mask
    full_vals = np.zeros((n, 3))
    full_vals[a.n_points:] = vals
    ref = O.DofMap(n, full_mask, full_vals)
    np.testing.assert_array_equal(dm.free_indices.numpy(), ref.free_indices)
    np.testing.assert_array_equal(dm.fixed_indices.numpy(), ref.fixed_indices)

    free = rng.normal(size=dm.n_free)
    full = dm.to_full(torch.as_tensor(free))
    np.testing.assert_array_equal(full.numpy(), ref.to_full(free))
    np.testing.assert_array_equal(dm.to_free(full).numpy(), free)
    np.testing.assert_array_equal(dm.to_full_grad(torch.as_tensor(free)).numpy(), ref.to_full_grad(free))


def test_fixed_values_outside_the_mask_are_ignored():
    m = meshgen.grid(2, 2, 2)
    bld = DofMapBuilder()
    bld.add_vertices(m)
    mask = np.zeros((m.n_points, 3), bool)
    mask[0] = (True, False, True)
    m.point_data["FixedMask"] = mask
    m.point_data["FixedValue"] = np.full((m.n_points, 3), 7.0)
    bld.add_fixed(m)
    dm = bld.finalize(dtype=torch.float64, device="cpu")
    np.testing.assert_array_equal(dm.fixed_indices.numpy(), [0, 2])
    full = dm.to_full(torch.zeros(dm.n_free, dtype=torch.float64))
    assert full[0, 0] == 7.0 and full[0, 1] == 0.0 and full[0, 2] == 7.0
    assert float(full[1:].abs().sum()) == 0.0
