"""apple_gb300: GB300-native FEM elasticity / PNCG hot path of liblaf/apple.

Host side in Python (this package) over hand-written sm_103a CUDA kernels in
``libapple_gb300.so`` (C ABI: ``include/apple_gb300.h``).
"""

from . import meshgen, vtu, warp
from .fem import Arap, Space, StableNeoHookean, StableNeoHookeanMuscle, WarpPotential, WarpPotentialFem, with_lame
from .forward import Forward, ForwardProblem, ModelState
from .model import DofMap, DofMapBuilder, Model, ModelBuilder, WarpModel
from .pncg import PNCG, ConvergenceCriteria, LineSearch, Result, Solution
from .potential import ExternalForce
from .region import Region

__all__ = [
    "Arap",
    "ConvergenceCriteria",
    "DofMap",
    "DofMapBuilder",
    "ExternalForce",
    "Forward",
    "ForwardProblem",
    "LineSearch",
    "Model",
    "ModelBuilder",
    "ModelState",
    "PNCG",
    "Region",
    "Result",
    "Solution",
    "Space",
    "StableNeoHookean",
    "StableNeoHookeanMuscle",
    "WarpModel",
    "WarpPotential",
    "WarpPotentialFem",
    "meshgen",
    "vtu",
    "warp",
    "with_lame",
]
