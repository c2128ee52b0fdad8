"""Multiphase (src/pmmoto/domain_generation/multiphase.py:18-130)."""

from __future__ import annotations

import numpy as np
import torch

from .. import _dev, _ops
from ..core.geometry import geo_of

__all__ = ["Multiphase"]


class Multiphase:
    """Phase image on a porous medium (0 solid, 1..num_phases fluids)."""

    def __init__(self, porous_media, img, num_phases: int):
        self.porous_media = porous_media
        self.pm_img = porous_media.img
        self.subdomain = porous_media.subdomain
        self.num_phases = num_phases
        self.img = img
        self.fluids = list(range(1, num_phases + 1))

    def update_img(self, img) -> None:
        """Reservoir voxels are set to phase 1 (:43-54)."""
        self.img = self.subdomain.update_reservoir(img, 1 if isinstance(img, torch.Tensor) else img.dtype.type(1))

    def get_volume_fraction(self, phase: int, img=None) -> float:
        """:56-80."""
        if img is None:
            img = self.img
        g = geo_of(self.subdomain)
        t, _ = _dev.to_device(img, torch.uint8)
        n = _ops.count_eq_device(t, _ops.box_of(g.own_box()), phase)
        return float(n / np.prod(self.subdomain.domain.voxels))

    def get_saturation(self, phase: int, img=None) -> float:
        """:82-96."""
        return self.get_volume_fraction(phase, img) / self.porous_media.porosity

    @staticmethod
    def get_probe_radius(pc: float, gamma: float = 1, contact_angle: float = 0) -> float:
        """:98-116."""
        if pc == 0:
            return 0
        return 2.0 * gamma / pc * np.cos(np.deg2rad(contact_angle))

    @staticmethod
    def get_pc(radius: float, gamma: float = 1) -> float:
        """:118-130."""
        return 2.0 * gamma / radius
