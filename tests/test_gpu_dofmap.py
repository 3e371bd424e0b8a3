"""The DOF-map kernels (``agb_dof_to_free`` / ``agb_dof_to_full``) against the
oracle's DofMap (forward/dof_map/_dof_map.py:30-50), bit for bit (GB300):
random masks, no fixed DOF, every DOF fixed."""

import numpy as np
import pytest
import torch

from apple_gb300.model import DofMap
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("frac", [0.0, 0.37, 1.0])
def test_dof_maps_match_the_oracle(dtype, frac, cuda_device):
    rng = np.random.default_rng(int(frac * 100))
    n = 1537
    mask = rng.random((n, 3)) < frac
    vals = rng.normal(size=(n, 3))
    dm = DofMap(n, mask, vals, device=cuda_device, dtype=dtype)
    ref = O.DofMap(n, mask, vals)
    free = rng.normal(size=dm.n_free)
    full = torch.as_tensor(rng.normal(size=(n, 3)), dtype=dtype, device=cuda_device)
    free_t = torch.as_tensor(free, dtype=dtype, device=cuda_device)
    np_dtype = np.float32 if dtype == torch.float32 else np.float64
    np.testing.assert_array_equal(dm.to_free(full).cpu().numpy(), full.cpu().numpy().reshape(-1)[ref.free_indices])
    got = dm.to_full(free_t).cpu().numpy()
    np.testing.assert_array_equal(got, ref.to_full(free.astype(np_dtype)).astype(np_dtype))
    got = dm.to_full_grad(free_t).cpu().numpy()
    np.testing.assert_array_equal(got, ref.to_full_grad(free.astype(np_dtype)).astype(np_dtype))
    # round trip
    np.testing.assert_array_equal(dm.to_free(dm.to_full(free_t)).cpu().numpy(), free_t.cpu().numpy())
