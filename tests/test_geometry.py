"""Host geometry of the package's single-rank subdomain vs the oracle's and
the reference's padding / feature rules (CPU only)."""

import itertools

import numpy as np
import pytest

from oracle import oracle as O
from pmmoto_gb300.core import initialize
from pmmoto_gb300.core.geometry import geo_of

KINDS = ["end", "wall", "periodic"]


@pytest.mark.parametrize("kinds", list(itertools.product(KINDS, repeat=3)))
def test_geometry_matches_oracle(kinds):
    bts = tuple((k, k) for k in kinds)
    vox = (7, 9, 11)
    box = ((0.0, 0.7), (0.1, 1.0), (-0.5, 0.6))
    inlet = ((kinds[0] == "end", False), (False, False), (False, False))
    outlet = ((False, kinds[0] == "end"), (False, False), (False, False))
    sd = initialize(vox, box=box, boundary_types=bts, inlet=inlet, outlet=outlet, reservoir_voxels=2)
    g = O.Geom(vox, boundary_types=bts, box=box, inlet=inlet, outlet=outlet, reservoir_voxels=2)
    assert sd.voxels == g.shape and sd.pad == g.pad and sd.reservoir_pad == g.reservoir_pad
    for a, b in zip(sd.coords, g.coords()):
        np.testing.assert_array_equal(a, b)
    geo = geo_of(sd)
    for f in O.ALL_FEATURES:
        btype, has_nb, own, nb = geo.feature(f)
        o_own, o_nb = g.feature_slabs(f)
        assert has_nb == g.feature_has_neighbor(f)
        assert tuple(slice(a, b) for a, b in own) == o_own
        assert tuple(slice(a, b) for a, b in nb) == o_nb
    img = np.ones(sd.voxels, np.uint8)
    np.testing.assert_array_equal(sd.set_wall_bcs(img.copy()), g.set_wall_bcs(img.copy()))
    np.testing.assert_array_equal(sd.update_reservoir(img.copy() * 0, 1), g.update_reservoir(img.copy() * 0, 1))
