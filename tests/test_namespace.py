"""The reference's import paths map one to one onto this package: the names
of liblaf.apple.forward (forward/__init__.pyi), liblaf.apple.warp.fem
(warp/fem/__init__.pyi), .warp.model (warp/model/__init__.pyi, without the
JAX FFI adapter), .warp.potential (warp/potential/__init__.pyi) and the
rotation-variant SVD / polar of .warp.math (warp/math/_rotation.py:9-22)."""

import numpy as np
import pytest

import apple_gb300 as ag
from apple_gb300 import forward
from apple_gb300.warp import fem, math, model, potential
from oracle import fem_oracle as O


def test_reference_names_exist():
    for name in ["DofMap", "DofMapBuilder", "Forward", "ForwardProblem", "Model", "ModelBuilder", "ModelState"]:
        assert hasattr(forward, name), name
    for name in ["Arap", "StableNeoHookean", "StableNeoHookeanMuscle", "WarpPotentialFem"]:
        assert hasattr(fem, name), name
    for name in ["WarpModel", "WarpPotential"]:
        assert hasattr(model, name), name
    assert hasattr(potential, "ExternalForce")
    for cls in (fem.Arap, fem.StableNeoHookean, fem.StableNeoHookeanMuscle, potential.ExternalForce):
        assert issubclass(cls, model.WarpPotential)


def test_base_potential_raises_not_implemented():
    p = ag.WarpPotential()
    with pytest.raises(NotImplementedError):
        p.fun(None, None)
    with pytest.raises(NotImplementedError):
        p.hess_prod(None, None, None)


def test_svd_rv_and_polar_rv():
    rng = np.random.default_rng(0)
    F = rng.normal(size=(200, 3, 3))
    F[:50] = np.eye(3) + 0.1 * F[:50]  # near the identity
    U, s, V = math.svd_rv(F)
    np.testing.assert_allclose(U @ (s[:, :, None] * np.swapaxes(V, 1, 2)), F, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(U), 1.0, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(V), 1.0, atol=1e-12)
    assert np.all(np.sign(s[:, 2]) == np.sign(np.linalg.det(F)))
    assert np.all(s[:, 0] >= s[:, 1]) and np.all(s[:, 1] >= np.abs(s[:, 2]))
    Uo, so, Vo = O.svd_rv(F)
    np.testing.assert_allclose(s, so, atol=1e-12)
    R, S = math.polar_rv(F)
    np.testing.assert_allclose(R @ S, F, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(R), 1.0, atol=1e-12)
    np.testing.assert_allclose(S, np.swapaxes(S, 1, 2), atol=1e-12)
    Ro, _ = O.polar_rv(F)
    np.testing.assert_allclose(R, Ro, atol=1e-10)
