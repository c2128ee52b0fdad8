"""Sphere lists with periodic images, ownership and trimming.

Same order of operations, same float64 tests and the same output order as
the reference's SphereList (src/pmmoto/particles/spheres.hpp):

* ``intersects_box`` (:56-64): not (c + r < min or c - r > max) on any axis;
* ``extends_outside_box`` (:95-106): c - r < min or c + r > max, per axis;
* ``inside_box`` (particle_list.hpp:56-61): min <= c <= max on every axis;
* ``add_periodic_spheres`` (:365-409): for every sphere and every shift
  dx, dy, dz in (-1, 0, 1) -- a nonzero shift only on an axis where the
  sphere extends outside the domain box and the axis is periodic -- the image
  c + shift * length is kept when it intersects the subdomain box (the
  unshifted sphere too), in loop order dx, dy, dz;
* ownership (``own_spheres`` :273-281) is "centre inside the own box".
"""

from __future__ import annotations

import numpy as np

from ..core.boundary_types import BoundaryType

__all__ = ["SphereList", "initialize_spheres"]


def _box(bounds):
    b = np.asarray(bounds, dtype=np.float64).reshape(3, 2)
    return b[:, 0].copy(), b[:, 1].copy()


def _intersects(c, r, lo, hi):
    return ~np.any((c + r[:, None] < lo) | (c - r[:, None] > hi), axis=1)


def _inside(c, lo, hi):
    return np.all((c >= lo) & (c <= hi), axis=1)


class SphereList:
    """x, y, z, r rows with an own flag (PySphereList, _particles.pyx:268-360)."""

    def __init__(self, coordinates, radii):
        c = np.asarray(coordinates, dtype=np.float64).reshape(-1, 3)
        if c.shape[0] == 0:
            raise ValueError("Cannot initialize PySphereList with empty coordinates")
        r = np.asarray(radii, dtype=np.float64).reshape(-1)
        if r.shape[0] != c.shape[0]:
            raise RuntimeError("Failed to create SphereList: coordinates and radii differ in length")
        self._c = c.copy()
        self._r = r.copy()
        self._own = np.zeros(c.shape[0], dtype=bool)
        self._own_count = 0

    def size(self) -> int:
        return int(self._c.shape[0])

    def get_own_count(self) -> int:
        return int(self._own_count)

    def return_coordinates(self):
        return self._c.copy()

    def return_np_array(self, return_own: bool = False):
        cols = [self._c, self._r[:, None]]
        if return_own:
            cols.append(self._own.astype(np.float64)[:, None])
        return np.concatenate(cols, axis=1)

    def _keep(self, mask):
        self._c, self._r, self._own = self._c[mask], self._r[mask], self._own[mask]

    def add_periodic(self, subdomain) -> None:
        """Periodic images crossing the domain boundary (spheres.hpp:365-409)."""
        dlo, dhi = _box(subdomain.domain.box)
        length = dhi - dlo
        periodic = np.array([subdomain.domain.boundary_types[d][0] == BoundaryType.PERIODIC and
                             subdomain.domain.boundary_types[d][1] == BoundaryType.PERIODIC for d in range(3)])
        slo, shi = _box(subdomain.box)
        ext = (self._c - self._r[:, None] < dlo) | (self._c + self._r[:, None] > dhi)
        out_c, out_r = [], []
        for k in range(self.size()):
            c, r = self._c[k], self._r[k]
            for dx in (-1, 0, 1):
                if dx != 0 and not (ext[k, 0] and periodic[0]):
                    continue
                for dy in (-1, 0, 1):
                    if dy != 0 and not (ext[k, 1] and periodic[1]):
                        continue
                    for dz in (-1, 0, 1):
                        if dz != 0 and not (ext[k, 2] and periodic[2]):
                            continue
                        img = c.copy()
                        img[0] += dx * length[0]
                        img[1] += dy * length[1]
                        img[2] += dz * length[2]
                        if not (img[0] + r < slo[0] or img[0] - r > shi[0] or img[1] + r < slo[1] or
                                img[1] - r > shi[1] or img[2] + r < slo[2] or img[2] - r > shi[2]):
                            out_c.append(img)
                            out_r.append(r)
        self._c = np.asarray(out_c, dtype=np.float64).reshape(-1, 3)
        self._r = np.asarray(out_r, dtype=np.float64)
        self._own = np.zeros(self._c.shape[0], dtype=bool)

    def set_own(self, subdomain) -> None:
        lo, hi = _box(subdomain.own_box)
        self._own = _inside(self._c, lo, hi)
        self._own_count = int(self._own.sum())

    def trim_intersecting(self, subdomain) -> None:
        lo, hi = _box(subdomain.box)
        self._keep(_intersects(self._c, self._r, lo, hi))

    def trim_within(self, subdomain) -> None:
        lo, hi = _box(subdomain.own_box)
        self._keep(_inside(self._c, lo, hi))


def initialize_spheres(subdomain, spheres, radii=None, add_periodic: bool = False, set_own: bool = True,
                       trim_intersecting: bool = False, trim_within: bool = False) -> SphereList:
    """initialize_spheres (particles.py:182-230)."""
    spheres = np.asarray(spheres, dtype=np.float64)
    if radii is None:
        coords, radii = spheres[:, 0:3], spheres[:, 3]
    else:
        coords = spheres
    particles = SphereList(coords, radii)
    if trim_intersecting:
        particles.trim_intersecting(subdomain)
    if trim_within:
        particles.trim_within(subdomain)
    if add_periodic and subdomain.domain.periodic_check():
        particles.add_periodic(subdomain)
    if set_own:
        particles.set_own(subdomain)
    return particles
