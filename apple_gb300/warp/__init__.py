"""The reference's ``liblaf.apple.warp`` namespace (warp/__init__.pyi):
``fem``, ``math``, ``model`` and ``potential``, mapped onto this package, so
``from liblaf.apple.warp import fem`` becomes ``from apple_gb300.warp import
fem`` with the same class names."""

from . import fem, math, model, potential

__all__ = ["fem", "math", "model", "potential"]
