"""Single-rank padded subdomain: the metadata the GPU path needs.

Restates, for one rank owning the whole domain, the geometry of
``pmmoto.initialize`` (src/pmmoto/core/pmmoto.py:20-80), ``Domain``
(core/domain.py), ``DiscretizedDomain`` (domain_discretization.py:56-90),
``PaddedSubdomain`` (subdomain_padded.py:21-307), ``Subdomain``
(subdomain.py:134-287), the feature slabs (features.py:76-139,
subdomain_features.py:60-158) and the neighbour map (domain_decompose.py:
62-100): with one rank only features whose every nonzero direction lies on a
periodic axis have a neighbour (rank 0 itself).

The MPI halo exchange of the reference becomes, on the device, index
arithmetic over these slabs; the host keeps only the bookkeeping here.
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np

from .boundary_types import BoundaryType, boundary_order, bt_value

FACES = [d for d in itertools.product(*[[-1, 0, 1]] * 3) if sum(abs(x) for x in d) == 1]
EDGES = [d for d in itertools.product([-1, 0, 1], repeat=3) if sum(abs(x) for x in d) == 2]
CORNERS = [(x, y, z) for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)]
ALL_FEATURES = FACES + EDGES + CORNERS  # orientation.py:40-183 iteration order


@dataclass
class Feature:
    feature_id: tuple
    boundary_type: BoundaryType
    neighbor_rank: int
    own: tuple  # ((lo, hi),) * 3
    neighbor: tuple
    inlet: bool = False
    outlet: bool = False

    @property
    def forward(self) -> bool:
        return not any(f == 1 for f in self.feature_id)

    @property
    def slice(self):
        sl = [slice(None)] * 3
        for d, f in enumerate(self.feature_id):
            if f == -1:
                sl[d] = 0
            elif f == 1:
                sl[d] = -1
        return tuple(sl)

    def own_slices(self):
        return tuple(slice(a, b) for a, b in self.own)

    def neighbor_slices(self):
        return tuple(slice(a, b) for a, b in self.neighbor)


def _slabs(fid, btype, shape, pad):
    padded = any(p for pp in pad for p in pp)
    own, nb = [], []
    for d in range(3):
        length = shape[d]
        pb, pa = pad[d]
        f = fid[d]
        if f == -1:
            own.append((pb, 2 * pb) if pb and btype != "wall" else (1, 2) if pb else (0, 1))
            nb.append(((0, 1) if btype == "wall" else (0, pb)) if padded else (0, 0))
        elif f == 1:
            own.append((length - 2 * pa, length - pa) if pa and btype != "wall"
                       else (length - 2, length - 1) if pa else (length - 1, length))
            nb.append(((length - 1, length) if btype == "wall" else (length - pa, length)) if padded else (0, 0))
        else:
            own.append((pb, length - pa))
            nb.append((pb, length - pa) if padded else (0, 0))
    return tuple(own), tuple(nb)


class Domain:
    """Global domain (box, boundaries, inlet/outlet, voxels, resolution)."""

    def __init__(self, box, boundary_types, inlet, outlet, voxels):
        self.box = tuple(tuple(float(x) for x in b) for b in box)
        # the box as given (the image writer prints it the way it came)
        self.box_input = tuple(tuple(b) for b in box)
        self.boundary_types = tuple(tuple(BoundaryType(bt_value(b)) for b in bt) for bt in boundary_types)
        self.inlet = inlet
        self.outlet = outlet
        self.dims = 3
        self.voxels = tuple(int(v) for v in voxels)
        self.subdomains = (1, 1, 1)
        self.num_subdomains = 1
        self.length = tuple(float(np.float64(b[1]) - np.float64(b[0])) for b in box)
        self.volume = float(np.prod(self.length))
        self.periodic = any(bt_value(b) == "periodic" for bt in self.boundary_types for b in bt)
        for n in range(3):
            if self.voxels[n] <= 1:
                raise AssertionError("every axis needs more than one voxel")
        self.resolution = tuple(self.length[n] / self.voxels[n] for n in range(3))

    def periodic_check(self) -> bool:
        return self.periodic


class PaddedSubdomain:
    """The one subdomain of a single-rank decomposition, with its halo."""

    def __init__(self, domain: Domain, pad=(1, 1, 1), reservoir_voxels: int = 0):
        self.rank = 0
        self.domain = domain
        self.index = (0, 0, 0)
        bts = [[bt_value(b) for b in bt] for bt in domain.boundary_types]
        self.pad = tuple((0 if bts[d][0] == "end" else 1 if bts[d][0] == "wall" else int(pad[d]),
                          0 if bts[d][1] == "end" else 1 if bts[d][1] == "wall" else int(pad[d]))
                         for d in range(3))
        self.inlet = tuple((bool(domain.inlet[d][0]) and bts[d][0] == "end",
                            bool(domain.inlet[d][1]) and bts[d][1] == "end") for d in range(3))
        self.outlet = tuple((bool(domain.outlet[d][0]) and bts[d][0] == "end",
                             bool(domain.outlet[d][1]) and bts[d][1] == "end") for d in range(3))
        if reservoir_voxels:
            self.reservoir_pad = tuple((reservoir_voxels if self.inlet[d][0] else 0,
                                        reservoir_voxels if self.inlet[d][1] else 0) for d in range(3))
        else:
            self.reservoir_pad = ((0, 0), (0, 0), (0, 0))
        self.own_voxels = domain.voxels
        self.voxels = tuple(domain.voxels[d] + sum(self.pad[d]) + sum(self.reservoir_pad[d]) for d in range(3))
        self.boundary_types = domain.boundary_types
        self.global_boundary = ((True, True),) * 3
        self.periodic = domain.periodic
        self.box = self._padded_box()
        self.own_box = self._own_box()
        self.coords = self._coords()
        self.start = tuple(-self.pad[d][0] - self.reservoir_pad[d][0] for d in range(3))
        self.features = _Features(self)

    # subdomain_padded.py:188-216
    def _own_box(self):
        box = []
        for d in range(3):
            length = self.own_voxels[d] * self.domain.resolution[d]
            lower = self.domain.box[d][1] - length
            box.append((lower, lower + length))
        return tuple(box)

    def _padded_box(self):
        box = []
        for d, (lo, hi) in enumerate(self._own_box()):
            res = self.domain.resolution[d]
            box.append((lo - (self.pad[d][0] + self.reservoir_pad[d][0]) * res,
                        hi + (self.pad[d][1] + self.reservoir_pad[d][1]) * res))
        return tuple(box)

    # domain_discretization.py:70-90
    def _coords(self):
        out = []
        for d in range(3):
            half = 0.5 * self.domain.resolution[d]
            out.append(np.linspace(self.box[d][0] + half, self.box[d][1] - half, self.voxels[d]))
        return out

    def get_own_voxels(self):
        own = np.zeros(6, dtype=np.int64)
        for d in range(3):
            own[2 * d] = self.pad[d][0] + self.reservoir_pad[d][0]
            own[2 * d + 1] = self.voxels[d] - self.pad[d][1] - self.reservoir_pad[d][1]
        return own

    def own_slices(self):
        o = self.get_own_voxels()
        return tuple(slice(int(o[2 * d]), int(o[2 * d + 1])) for d in range(3))

    def get_length(self):
        return tuple(self.box[d][1] - self.box[d][0] for d in range(3))

    def check_boundary_type(self, boundary_type) -> bool:
        v = bt_value(boundary_type)
        return any(bt_value(b) == v for bt in self.boundary_types for b in bt)

    def set_wall_bcs(self, img):
        """subdomain.py:273-287 (host arrays or CUDA tensors)."""
        for f in self.features.faces.values():
            if bt_value(f.boundary_type) == "wall":
                img[f.slice] = 0
        return img

    def update_reservoir(self, img, value):
        """subdomain_padded.py:285-307."""
        for d, (a, b) in enumerate(self.reservoir_pad):
            if a > 0:
                sl = [slice(None)] * 3
                sl[d] = slice(0, a)
                img[tuple(sl)] = value
            if b > 0:
                sl = [slice(None)] * 3
                sl[d] = slice(img.shape[d] - b, None)
                img[tuple(sl)] = value
        return img


class _Features:
    def __init__(self, sd: PaddedSubdomain):
        bts = [[bt_value(b) for b in bt] for bt in sd.boundary_types]
        self.faces, self.edges, self.corners = {}, {}, {}
        for fid in ALL_FEATURES:
            kinds = []
            for d in range(3):
                if fid[d] == -1:
                    kinds.append(bts[d][0])
                elif fid[d] == 1:
                    kinds.append(bts[d][1])
            btype = boundary_order(kinds)
            has_nb = all(fid[d] == 0 or bts[d][0] == "periodic" for d in range(3))
            own, nb = _slabs(fid, btype.value, sd.voxels, sd.pad)
            feat = Feature(fid, btype, 0 if has_nb else (-2 if btype == BoundaryType.WALL else -1), own, nb)
            if fid in FACES:
                d = [i for i in range(3) if fid[i] != 0][0]
                side = 0 if fid[d] < 0 else 1
                feat.inlet = sd.inlet[d][side]
                feat.outlet = sd.outlet[d][side]
                self.faces[fid] = feat
            elif fid in EDGES:
                self.edges[fid] = feat
            else:
                self.corners[fid] = feat

    @property
    def all_features(self):
        yield from self.faces.items()
        yield from self.edges.items()
        yield from self.corners.items()


def initialize(voxels, box=((0, 1.0), (0, 1.0), (0, 1)), subdomains=(1, 1, 1),
               boundary_types=((BoundaryType.END, BoundaryType.END),) * 3,
               inlet=((False, False),) * 3, outlet=((False, False),) * 3, reservoir_voxels=0,
               rank=0, pad=(1, 1, 1), verlet_domains=(1, 1, 1), return_subdomain=False):
    """pmmoto.initialize (core/pmmoto.py:20-80) for one rank on one GPU."""
    if tuple(subdomains) != (1, 1, 1) or rank != 0:
        raise NotImplementedError("pmmoto_gb300 runs the whole domain as one subdomain on one GPU")
    dom = Domain(box, boundary_types, inlet, outlet, voxels)
    return PaddedSubdomain(dom, pad=pad, reservoir_voxels=reservoir_voxels)
