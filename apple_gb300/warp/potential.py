"""``liblaf.apple.warp.potential`` (warp/potential/__init__.pyi)."""

from ..potential import ExternalForce

__all__ = ["ExternalForce"]
