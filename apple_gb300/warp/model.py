"""``liblaf.apple.warp.model`` (warp/model/__init__.pyi): the energy-term
interface and the model sum.  (``WarpModelAdapter``, the JAX FFI glue, has
no counterpart: the potentials take torch tensors directly.)"""

from ..fem import WarpPotential
from ..model import WarpModel

__all__ = ["WarpModel", "WarpPotential"]
