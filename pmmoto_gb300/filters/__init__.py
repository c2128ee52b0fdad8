"""GPU drop-ins for ``pmmoto.filters``."""

from . import distance  # noqa: F401

__all__ = ["distance"]
