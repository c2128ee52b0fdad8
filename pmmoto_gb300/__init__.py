"""pmmoto_gb300 -- GB300-native voxel-morphology path of PMMoTo.

A drop-in for the reference's hot path (``pmmoto.filters.distance``,
``pmmoto.filters.morphological_operators``, ``pmmoto.filters.connected_components``,
``pmmoto.filters.porosimetry``, ``pmmoto.filters.equilibrium_distribution`` and
``pmmoto.domain_generation.gen_pm_spheres_domain``): Python host code calls
hand-written sm_103a CUDA kernels through the C ABI in
``include/pmmoto_gb300.h``, one subdomain on one GPU.
"""

from . import core, domain_generation, filters, io, particles  # noqa: F401
from .core import BoundaryType, initialize  # noqa: F401

__all__ = ["initialize", "BoundaryType", "core", "domain_generation", "filters", "io", "particles"]
