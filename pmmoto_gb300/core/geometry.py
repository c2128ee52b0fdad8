"""Flat geometry record read from any single-rank subdomain object.

Accepts this package's ``PaddedSubdomain`` or the reference's
(``pmmoto.core.subdomain_padded.PaddedSubdomain`` / ``VerletSubdomain``):
both expose ``voxels``, ``pad``, ``reservoir_pad``, ``inlet``, ``outlet``,
``own_voxels`` and ``domain.{boundary_types, resolution, periodic}``.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .boundary_types import bt_value
from .subdomain import ALL_FEATURES, FACES, _slabs
from .boundary_types import boundary_order

BC_CODE = {"end": 0, "wall": 1, "periodic": 2}


@dataclass
class Geo:
    shape: tuple
    pad: tuple
    rpad: tuple
    bts: tuple
    inlet: tuple
    outlet: tuple
    res: tuple
    own_voxels: tuple
    domain_voxels: tuple

    @property
    def periodic(self) -> bool:
        return any(b == "periodic" for bt in self.bts for b in bt)

    def axis_periodic(self, d) -> bool:
        return self.bts[d][0] == "periodic"

    def bc_codes(self) -> np.ndarray:
        return np.ascontiguousarray([BC_CODE[self.bts[d][s]] for d in range(3) for s in (0, 1)], dtype=np.int32)

    def pad_flat(self) -> np.ndarray:
        return np.ascontiguousarray([self.pad[d][s] for d in range(3) for s in (0, 1)], dtype=np.int32)

    def own_box(self):
        return tuple((self.pad[d][0] + self.rpad[d][0], self.shape[d] - self.pad[d][1] - self.rpad[d][1])
                     for d in range(3))

    def feature(self, fid):
        kinds = []
        for d in range(3):
            if fid[d] == -1:
                kinds.append(self.bts[d][0])
            elif fid[d] == 1:
                kinds.append(self.bts[d][1])
        btype = boundary_order(kinds).value
        has_nb = all(fid[d] == 0 or self.bts[d][0] == "periodic" for d in range(3))
        own, nb = _slabs(fid, btype, self.shape, self.pad)
        return btype, has_nb, own, nb

    def periodic_features(self):
        """Features with a (self) neighbour, in the reference's iteration order."""
        return [f for f in ALL_FEATURES if self.feature(f)[1]]

    def face_slab(self, which: str):
        """Own slab of the last inlet (or outlet) face in face order
        (voxels.py:400-454 overwrite earlier faces), or None."""
        flags = self.inlet if which == "inlet" else self.outlet
        slab = None
        for f in FACES:
            d = [i for i in range(3) if f[i] != 0][0]
            side = 0 if f[d] < 0 else 1
            if flags[d][side]:
                slab = self.feature(f)[2]
        return slab


def geo_of(sd) -> Geo:
    if getattr(sd.domain, "num_subdomains", 1) > 1:
        raise NotImplementedError("pmmoto_gb300 runs one subdomain per GPU")
    bts = tuple(tuple(bt_value(b) for b in bt) for bt in sd.domain.boundary_types)
    rpad = tuple(tuple(int(x) for x in p) for p in getattr(sd, "reservoir_pad", ((0, 0),) * 3))
    return Geo(shape=tuple(int(v) for v in sd.voxels), pad=tuple(tuple(int(x) for x in p) for p in sd.pad),
               rpad=rpad, bts=bts, inlet=tuple(tuple(bool(x) for x in i) for i in sd.inlet),
               outlet=tuple(tuple(bool(x) for x in o) for o in sd.outlet),
               res=tuple(float(r) for r in sd.domain.resolution),
               own_voxels=tuple(int(v) for v in sd.own_voxels), domain_voxels=tuple(int(v) for v in sd.domain.voxels))
