"""``liblaf.apple.warp.fem`` (warp/fem/__init__.pyi): the FEM potentials."""

from ..fem import Arap, StableNeoHookean, StableNeoHookeanMuscle, WarpPotentialFem

__all__ = ["Arap", "StableNeoHookean", "StableNeoHookeanMuscle", "WarpPotentialFem"]
