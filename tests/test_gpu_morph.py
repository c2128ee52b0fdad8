"""Erode / dilate parity: CUDA path vs the reference fixtures and the oracle."""

import itertools

import numpy as np
import pytest

from oracle import oracle as O
from tests._helpers import geom_from_meta, sd_from_meta

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    from pmmoto_gb300.filters import morphological_operators
    return morphological_operators


@pytest.mark.parametrize("ci", range(5))
def test_morph_golden(M, golden, golden_meta, ci):
    case = golden_meta["sub_cases"][ci]
    sd = sd_from_meta(case["geom"])
    img = golden[f"sub_{ci}_img"]
    for ri, r in enumerate(case["radii"]):
        np.testing.assert_array_equal(M.erode(sd, img, r), golden[f"sub_{ci}_erode_{ri}"])
        np.testing.assert_array_equal(M.dilate(sd, img, r), golden[f"sub_{ci}_dilate_{ri}"])
        np.testing.assert_array_equal(M.erode(sd, img, np.float64(r)), golden[f"sub_{ci}_erode64_{ri}"])
        np.testing.assert_array_equal(M.erode(sd, img, r, fft=True), golden[f"sub_{ci}_erodefft_{ri}"])
        np.testing.assert_array_equal(M.dilate(sd, img, r, fft=True), golden[f"sub_{ci}_dilatefft_{ri}"])


@pytest.mark.parametrize("kinds", list(itertools.product(["end", "wall", "periodic"], repeat=3))[::2])
@pytest.mark.parametrize("scale", [20, 16])
def test_morph_random_vs_oracle(M, kinds, scale):
    """scale 16 gives power-of-two voxels (1/16), which take the exact integer
    passes; radii 0.125 and 0.1875 are then exactly 2 and 3 voxels (ties)."""
    rng = np.random.default_rng(sum(map(ord, "".join(kinds))))
    vox = (20, 17, 23)
    box = tuple((0.0, v / scale) for v in vox)
    bts = tuple((k, k) for k in kinds)
    from pmmoto_gb300.core import initialize
    sd = initialize(vox, box=box, boundary_types=bts)
    g = O.Geom(vox, boundary_types=bts, box=box)
    img = (rng.random(sd.voxels) > 0.3).astype(np.uint8)
    img = O.update_buffer(g, img)
    for r in (0.05, 0.1, np.float64(0.15), 0.24, 0.125, np.float64(0.1875)):
        if r < 1.0 / scale:
            continue  # the reference rejects radii below the voxel size
        np.testing.assert_array_equal(M.erode(sd, img, r), O.erode(g, img, r))
        np.testing.assert_array_equal(M.dilate(sd, img, r), O.dilate(g, img, r))
    np.testing.assert_array_equal(M.opening(sd, img, 0.1), O.opening(g, img, 0.1))
    np.testing.assert_array_equal(M.closing(sd, img, 0.1), O.closing(g, img, 0.1))


def test_morph_errors(M):
    from pmmoto_gb300.core import initialize
    sd = initialize((10, 10, 10), boundary_types=(("periodic",) * 2,) * 3)
    img = np.ones(sd.voxels, np.uint8)
    with pytest.raises(ValueError):
        M.erode(sd, img, 0.01)  # radius below the resolution
    with pytest.raises(SystemExit):
        M.erode(sd, img, 1.5)  # extension beyond the subdomain


@pytest.mark.parametrize("kinds", [("wall", "wall", "wall"), ("end", "periodic", "wall"), ("periodic", "end", "end"),
                                   ("wall", "end", "periodic")])
@pytest.mark.parametrize("vox", [(36, 35, 38), (37, 40, 36), (39, 36, 37)])
def test_morph_window_widths_vs_oracle(M, kinds, vox):
    """Power-of-two voxels (1/32) with radii of W + 1/2 voxels, W = 0 .. 21:
    the integer passes take direct minima on line pairs for W <= 20 when the
    contiguous extent is even, the parabola envelope otherwise."""
    rng = np.random.default_rng(7 + sum(vox) + sum(map(ord, "".join(kinds))))
    scale = 32
    box = tuple((0.0, v / scale) for v in vox)
    bts = tuple((k, k) for k in kinds)
    from pmmoto_gb300.core import initialize
    sd = initialize(vox, box=box, boundary_types=bts)
    g = O.Geom(vox, boundary_types=bts, box=box)
    # a few seeds for the dilation, a few holes for the erosion
    few = np.zeros(sd.voxels, np.uint8)
    few[tuple(rng.integers(0, v, 6) for v in sd.voxels)] = 1
    sparse = O.update_buffer(g, few)
    dense = O.update_buffer(g, 1 - few)
    for w in range(0, 22):
        r = (w + 0.5) / scale
        if r < 1.0 / scale:
            continue  # the reference rejects radii below the voxel size
        np.testing.assert_array_equal(M.dilate(sd, sparse, r), O.dilate(g, sparse, r), err_msg=f"dilate W={w}")
        np.testing.assert_array_equal(M.erode(sd, dense, r), O.erode(g, dense, r), err_msg=f"erode W={w}")
