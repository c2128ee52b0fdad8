"""Sphere lists for voxelisation: drop-in for ``pmmoto.particles``'s sphere
part (src/pmmoto/particles/particles.py:182-230, _particles.pyx:268-360,
spheres.hpp:41-64, 249-409), host side -- the voxelisation itself runs on the
GPU (``domain_generation.gen_pm_shape``)."""

from .particles import SphereList, initialize_spheres  # noqa: F401

__all__ = ["SphereList", "initialize_spheres"]
