"""GPU drop-ins for ``pmmoto.filters``."""

from . import connected_components, distance, equilibrium_distribution, morphological_operators, porosimetry  # noqa: F401

__all__ = ["morphological_operators", "connected_components", "distance", "porosimetry", "equilibrium_distribution"]
