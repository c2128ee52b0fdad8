"""Sphere-pack porous media and constant multiphase images
(src/pmmoto/domain_generation/domain_generation.py:125-155, 290-306)."""

from __future__ import annotations

import numpy as np
import torch

from .. import _dev, _ops
from ..core.geometry import geo_of
from . import multiphase, porousmedia

__all__ = ["gen_pm_spheres_domain", "gen_pm_shape", "gen_mp_constant"]


def gen_pm_spheres_domain(subdomain, spheres, kd: bool = False, invert: bool = False):
    """Voxelise spheres (x, y, z, r rows) on the padded subdomain: pore = 1
    outside every sphere; then halo update, optional inversion, wall rule.
    ``kd`` selected the reference's kd-tree search, which gives the same image
    as the brute-force test; both map to the same kernel here."""
    g = geo_of(subdomain)
    t = _ops.spheres_device(spheres, subdomain.coords)
    if tuple(t.shape) != g.shape:
        raise ValueError("subdomain coords do not match its voxels")
    _ops.update_buffer_device(t, g)
    if invert:
        t = (t == 0).to(torch.uint8)
    img = t if isinstance(spheres, torch.Tensor) else t.cpu().numpy()
    img = subdomain.set_wall_bcs(img)
    return porousmedia.gen_pm(subdomain, img)


def gen_pm_shape(subdomain, shapes, kd: bool = False):
    """gen_pm_shape (_domain_generation.pyx:30-92) for a sphere list (from
    ``particles.initialize_spheres``, periodic images included) or an (N, 4)
    array: 1 at voxel centres outside every sphere, 0 inside; no halo update
    and no wall rule.  numpy arrays / lists give numpy, CUDA tensors stay on
    the device."""
    arr = shapes.return_np_array() if hasattr(shapes, "return_np_array") else shapes
    g = geo_of(subdomain)
    t = _ops.spheres_device(arr, subdomain.coords)
    if tuple(t.shape) != g.shape:
        raise ValueError("subdomain coords do not match its voxels")
    return t if isinstance(arr, torch.Tensor) else t.cpu().numpy()


def gen_mp_constant(porous_media, fluid_phase: int = 1):
    """All pore voxels set to one fluid phase (:290-306)."""
    img = porous_media.img
    if isinstance(img, torch.Tensor):
        mp_img = torch.where(img == 1, fluid_phase, 0).to(torch.uint8)
    else:
        mp_img = np.where(img == 1, fluid_phase, 0).astype(np.uint8)
    return multiphase.Multiphase(porous_media, mp_img, 2)
