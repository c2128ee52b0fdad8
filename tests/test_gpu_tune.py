"""The autotuner on the GPU: every candidate of every EDT knob gives the same
bits (the knobs change launch shapes, never results), tuning a shape class
picks candidates from the lists and caches them, and apply() sets them in
the library; the PMG_TUNE override wins over the cache."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_every_candidate_gives_the_same_bits():
    from pmmoto_gb300 import tune
    from pmmoto_gb300.filters import distance as D

    rng = np.random.default_rng(41)
    img = (rng.random((96, 70, 130)) >= 0.2).astype(np.uint8)
    per = (True, True, False)
    want = O.edt3d(img, periodic=per, squared=True)
    try:
        for name, cands in tune.KNOBS["edt"].items():
            for c in cands:
                tune._set_lib(name, c)
                np.testing.assert_array_equal(D.edt3d(img, periodic=per, squared=True), want)
            tune._set_lib(name, 0)
    finally:
        for name in tune.KNOBS["edt"]:
            tune._set_lib(name, 0)


def _wide_pore_media():
    """Media whose distances run past the windowed passes' +-12 window: a few
    scattered solid voxels, and solid balls of radius 4-9 at porosity ~0.8."""
    rng = np.random.default_rng(43)
    shape = (96, 80, 128)
    sparse = (rng.random(shape) >= 2e-4).astype(np.uint8)
    balls = np.ones(shape, np.uint8)
    idx = np.indices(shape)
    for _ in range(40):
        c = rng.random(3) * shape
        r = rng.uniform(4, 9)
        balls[((idx - c[:, None, None, None]) ** 2).sum(0) <= r * r] = 0
    return [sparse, balls]


@pytest.mark.parametrize("per", [(True, True, True), (True, False, True), (False, False, False)])
def test_envelope_paths_agree_on_wide_pores(per):
    """The windowed passes with the +-12, +-8 and (strided) +-24 windows
    (deferred voxels scanned past the window), the same passes handed to the
    float envelope by the probe, the exact integer stream and the float
    envelope give the oracle's bits."""
    from pmmoto_gb300 import tune
    from pmmoto_gb300.filters import distance as D

    names = ("edt.path", "edt.fallback", "edt.fallback_rows", "edt.narrow", "edt.narrow_rows", "edt.wide")
    try:
        for img in _wide_pore_media():
            want = O.edt3d(img, periodic=per, squared=True)
            assert want.max() > 14 ** 2  # the scans pass the window
            for path, thr, narrow, wide in ((0, 8193, 0, 0), (0, 8193, 8193, 0), (0, 0, 0, 0), (0, 0, 0, 8193),
                                            (1, 8193, 0, 0), (2, 8193, 0, 0)):
                for name, v in zip(names, (path, thr, thr, narrow, narrow, wide)):
                    tune._set_lib(name, v)
                np.testing.assert_array_equal(D.edt3d(img, periodic=per, squared=True), want,
                                              err_msg=f"path {path} fallback {thr} narrow {narrow} wide {wide}")
    finally:
        for name in names:
            tune._set_lib(name, -1)


@pytest.mark.parametrize("kinds,p", [(("periodic",) * 3, 0.35), (("end", "wall", "periodic"), 0.6),
                                     (("end",) * 3, 0.8)])
def test_cross_tile_and_seam_variants_give_the_same_labels(kinds, p):
    from pmmoto_gb300 import tune
    from pmmoto_gb300.core import initialize
    from pmmoto_gb300.filters import connected_components as C

    vox = (70, 40, 130)
    bts = tuple((k, k) for k in kinds)
    sd = initialize(vox, box=tuple((0.0, v / 64) for v in vox), boundary_types=bts)
    g = O.Geom(vox, boundary_types=bts, box=tuple((0.0, v / 64) for v in vox))
    rng = np.random.default_rng(7)
    img = O.update_buffer(g, (rng.random(sd.voxels) < p).astype(np.uint8))
    want, wn = O.connect_components(img, g)
    try:
        for fused, batched in ((0, 1), (1, 1), (0, 0)):
            tune._set_lib("cc.cross_fused", fused)
            tune._set_lib("cc.seam_batched", batched)
            lbl, n = C.connect_components(img, sd)
            np.testing.assert_array_equal(lbl, want)
            assert n == wn
    finally:
        tune.reset_lib("cc")
        tune._set_lib("cc.seam_batched", -1)


def test_tune_cache_apply_and_override(tmp_path, monkeypatch):
    from pmmoto_gb300 import tune

    monkeypatch.setenv("PMG_TUNE_CACHE", str(tmp_path / "t.json"))
    monkeypatch.delenv("PMG_TUNE", raising=False)
    try:
        best = tune.tune_edt((64, 64, 64), steps=1, force=True)
        for name, v in best.items():
            assert v in tune.KNOBS["edt"][name]
            assert tune.get_lib(name) == v
        assert tune.load_cache()[tune.key("edt", (64, 64, 64))]["settings"] == best
        monkeypatch.setenv("PMG_TUNE", "edt.rows_ctas=4")
        tune._applied.clear()
        assert tune.apply("edt", (64, 64, 64))["edt.rows_ctas"] == 4
        assert tune.get_lib("edt.rows_ctas") == 4
    finally:
        tune._applied.clear()
        for name in tune.KNOBS["edt"]:
            tune._set_lib(name, 0)
