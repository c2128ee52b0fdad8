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


@pytest.mark.parametrize("kinds,p", [(("periodic",) * 3, 0.35), (("end", "wall", "periodic"), 0.6),
                                     (("end",) * 3, 0.8)])
def test_cross_tile_variants_give_the_same_labels(kinds, p):
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
        for fused in (0, 1):
            tune._set_lib("cc.cross_fused", fused)
            lbl, n = C.connect_components(img, sd)
            np.testing.assert_array_equal(lbl, want)
            assert n == wn
    finally:
        tune.reset_lib("cc")


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
