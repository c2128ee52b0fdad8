"""Connected components parity: CUDA path vs the reference fixtures and the oracle."""

import itertools

import numpy as np
import pytest

from oracle import oracle as O
from tests._helpers import sd_from_meta

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def C():
    from pmmoto_gb300.filters import connected_components
    return connected_components


@pytest.mark.parametrize("ci", range(8))
def test_cc_golden(C, golden, golden_meta, ci):
    case = golden_meta["cc_cases"][ci]
    sd = sd_from_meta(case["geom"])
    lbl, n = C.connect_components(golden[f"cc_{ci}_in"], sd)
    np.testing.assert_array_equal(lbl, golden[f"cc_{ci}_out"])
    assert n == case["count"]


@pytest.mark.parametrize("ci", range(5))
def test_cc_sub_golden(C, golden, golden_meta, ci):
    case = golden_meta["sub_cases"][ci]
    lbl, n = C.connect_components(golden[f"sub_{ci}_img"], sd_from_meta(case["geom"]))
    np.testing.assert_array_equal(lbl, golden[f"sub_{ci}_cc"])
    assert n == case["cc_count"]


def test_selection_golden(C, golden, golden_meta):
    sd = sd_from_meta(golden_meta["drain_geom"])
    img = golden["drain_img"]
    np.testing.assert_array_equal(C.inlet_connected_img(sd, img), golden["drain_inlet_img"])
    np.testing.assert_array_equal(C.outlet_connected_img(sd, img), golden["drain_outlet_img"])
    np.testing.assert_array_equal(C.inlet_outlet_connected_img(sd, img), golden["drain_io_img"])
    np.testing.assert_array_equal(C.isolated_img(sd, img), golden["drain_iso_img"])


@pytest.mark.parametrize("kinds", list(itertools.product(["end", "wall", "periodic"], repeat=3))[1::3])
def test_cc_random_vs_oracle(C, kinds):
    from pmmoto_gb300.core import initialize
    rng = np.random.default_rng(sum(map(ord, "".join(kinds))) + 5)
    vox = (19, 13, 22)
    bts = tuple((k, k) for k in kinds)
    inlet = ((kinds[0] == "end", False), (False, False), (False, False))
    outlet = ((False, kinds[0] == "end"), (False, False), (False, False))
    box = tuple((0.0, v / 20) for v in vox)
    sd = initialize(vox, box=box, boundary_types=bts, inlet=inlet, outlet=outlet)
    g = O.Geom(vox, boundary_types=bts, box=box, inlet=inlet, outlet=outlet)
    for p in (0.35, 0.55, 0.8):
        img = O.update_buffer(g, (rng.random(sd.voxels) < p).astype(np.uint8))
        lbl, n = C.connect_components(img, sd)
        want, wn = O.connect_components(img, g)
        np.testing.assert_array_equal(lbl, want)
        assert n == wn
        # one nonzero value other than 1 (block labelling) and several values
        # (voxel labelling)
        single = (3 * img).astype(np.uint8)
        lbl, n = C.connect_components(single, sd)
        want, wn = O.connect_components(single, g)
        np.testing.assert_array_equal(lbl, want)
        assert n == wn
        multi = O.update_buffer(g, rng.integers(0, 3, sd.voxels).astype(np.uint8))
        lbl, n = C.connect_components(multi, sd)
        want, wn = O.connect_components(multi, g)
        np.testing.assert_array_equal(lbl, want)
        assert n == wn
        for phase in (None, 1, 2):
            np.testing.assert_array_equal(C.inlet_connected_img(sd, multi, phase), O.inlet_connected_img(g, multi, phase))
            np.testing.assert_array_equal(C.outlet_connected_img(sd, multi, phase), O.outlet_connected_img(g, multi, phase))
            np.testing.assert_array_equal(C.isolated_img(sd, multi, phase), O.isolated_img(g, multi, phase))


def test_cc_determinism(C):
    """Two runs on the same input give identical labels (no race in the numbering)."""
    from pmmoto_gb300.core import initialize
    sd = initialize((64, 64, 64), boundary_types=(("periodic",) * 2,) * 3)
    rng = np.random.default_rng(9)
    img = (rng.random(sd.voxels) < 0.3).astype(np.uint8)
    a, n1 = C.connect_components(img, sd)
    b, n2 = C.connect_components(img, sd)
    np.testing.assert_array_equal(a, b)
    assert n1 == n2


@pytest.mark.parametrize("kinds", [("end", "end", "end"), ("periodic", "wall", "periodic"), ("periodic",) * 3])
def test_cc_many_tiles_vs_oracle(C, kinds):
    """Volumes spanning many 4x8x32 labelling tiles in every direction."""
    from pmmoto_gb300.core import initialize
    rng = np.random.default_rng(77)
    vox = (37, 45, 101)
    bts = tuple((k, k) for k in kinds)
    box = tuple((0.0, v / 64) for v in vox)
    sd = initialize(vox, box=box, boundary_types=bts)
    g = O.Geom(vox, boundary_types=bts, box=box)
    for p in (0.3, 0.6):
        img = O.update_buffer(g, (rng.random(sd.voxels) < p).astype(np.uint8))
        lbl, n = C.connect_components(img, sd)
        want, wn = O.connect_components(img, g)
        np.testing.assert_array_equal(lbl, want)
        assert n == wn


@pytest.mark.parametrize("kinds", [("end", "wall", "wall"), ("end", "periodic", "periodic"), ("end", "end", "periodic")])
@pytest.mark.parametrize("vox", [(33, 27, 41), (21, 37, 141), (5, 6, 2200)])
def test_binary_block_selection_vs_oracle(C, kinds, vox):
    """The 2x2x2-block selection (phase filter, or the binary flag) equals the
    voxel-level selection of the reference, odd sizes included; the second
    shape spans several 8 x 16 x 64-voxel tiles on every axis, the third has
    rows longer than 2048 voxels."""
    import torch
    from pmmoto_gb300.core import initialize
    from pmmoto_gb300.core.geometry import geo_of
    rng = np.random.default_rng(5)
    bts = tuple((k, k) for k in kinds)
    inlet, outlet = ((True, False), (False, False), (False, False)), ((False, True), (False, False), (False, False))
    box = tuple((0.0, v / 64) for v in vox)
    sd = initialize(vox, box=box, boundary_types=bts, inlet=inlet, outlet=outlet)
    g = O.Geom(vox, boundary_types=bts, box=box, inlet=inlet, outlet=outlet)
    for p in (0.35, 0.5, 0.7):
        img = O.update_buffer(g, (rng.random(sd.voxels) < p).astype(np.uint8))
        t = torch.as_tensor(img, device="cuda")
        for mode, fn in ((C.SEL_INLET, O.inlet_connected_img), (C.SEL_OUTLET, O.outlet_connected_img),
                         (C.SEL_BOTH, O.inlet_outlet_connected_img), (C.SEL_ISOLATED, O.isolated_img)):
            got = C.select_device(geo_of(sd), t, mode | C.SEL_BINARY).cpu().numpy()
            np.testing.assert_array_equal(got, fn(g, img).astype(np.uint8))
        multi = O.update_buffer(g, rng.integers(0, 3, sd.voxels).astype(np.uint8))
        for phase in (1, 2):
            np.testing.assert_array_equal(C.outlet_connected_img(sd, multi, phase), O.outlet_connected_img(g, multi, phase))
