"""PorousMedia (src/pmmoto/domain_generation/porousmedia.py:18-118)."""

from __future__ import annotations

import numpy as np
import torch

from .. import _dev, _ops
from ..core.geometry import geo_of

__all__ = ["PorousMedia", "gen_pm"]


class PorousMedia:
    """Binary porous medium (1 = pore) on a subdomain, with cached porosity
    and distance transform."""

    def __init__(self, subdomain, img):
        self.subdomain = subdomain
        self.img = img
        self._porosity = None
        self._distance = None
        self._max_distance = None

    @property
    def porosity(self) -> float:
        if self._porosity is None:
            self.set_porosity()
        return self._porosity

    def set_porosity(self) -> None:
        """Own-region pore count over the domain voxel count (:53-66)."""
        g = geo_of(self.subdomain)
        t, _ = _dev.to_device(self.img, torch.uint8)
        n = _ops.count_eq_device(t, _ops.box_of(g.own_box()), 1)
        self._porosity = n / np.prod(self.subdomain.domain.voxels)

    @property
    def distance(self):
        if self._distance is None:
            self.set_distance()
        return self._distance

    @property
    def max_distance(self) -> float:
        """determine_maximum of the halo-updated distance (:82-94)."""
        if self._max_distance is None:
            d = self.distance
            t = d if isinstance(d, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(d)).cuda()
            self._max_distance = _ops.max_f32_device(t)
        return self._max_distance

    def set_distance(self) -> None:
        """edt(img, subdomain) followed by update_buffer (:96-101)."""
        from ..filters import distance

        g = geo_of(self.subdomain)
        t, kind = _dev.to_device(self.img, torch.uint8)
        if g.periodic:
            d = distance.edt3d_device(t, distance._res32(g.res, 3), distance.padded_cfg(g.pad, [g.axis_periodic(k) for k in range(3)]), False)
        else:
            d = distance.edt3d_device(t, distance._res32(g.res, 3), distance.edt3d_cfg((False,) * 3), False)
        _ops.update_buffer_device(d, g)
        self._distance = _dev.give_back(d, kind)


def gen_pm(subdomain, img) -> PorousMedia:
    """porousmedia.py:104-118."""
    return PorousMedia(subdomain=subdomain, img=img)
