"""Host logic of the autotuner: shape classes, cache keys and round trips,
the PMG_TUNE override, and the library's tunable-parameter table (names,
ranges, defaults) -- no GPU needed."""

import ctypes
import json

import pytest

from pmmoto_gb300 import tune


def test_shape_class_and_key():
    assert tune.shape_class((1024, 1026, 3)) == "1024x2048x4"
    assert tune.key("edt", (96, 128, 130), gpu="G") == "G|edt|128x128x256"


def test_cache_round_trip_and_override(tmp_path, monkeypatch):
    monkeypatch.setenv("PMG_TUNE_CACHE", str(tmp_path / "c.json"))
    monkeypatch.delenv("PMG_TUNE", raising=False)
    k = tune.key("edt", (64, 64, 64), gpu="cpu")
    tune.save_entry(k, {"edt.pair_seg": 512}, {"edt.pair_seg": {"512": 1.0}})
    assert json.load(open(tmp_path / "c.json"))[k]["settings"] == {"edt.pair_seg": 512}
    monkeypatch.setattr(tune, "gpu_name", lambda: "cpu")
    assert tune.settings_for("edt", (60, 64, 33)) == {"edt.pair_seg": 512}
    monkeypatch.setenv("PMG_TUNE", "edt.pair_seg=128, edt.rows_ctas=8")
    assert tune.settings_for("edt", (64, 64, 64)) == {"edt.pair_seg": 128, "edt.rows_ctas": 8}
    monkeypatch.setenv("PMG_TUNE", "edt.pair_seg")
    with pytest.raises(ValueError):
        tune.overrides()


def test_library_knob_table():
    from pmmoto_gb300 import _lib

    L = _lib.lib()
    v = ctypes.c_int32(0)
    for name, cands in tune.KNOBS["edt"].items():
        assert L.pmg_tune_get(name.encode(), ctypes.byref(v)) == 0
        default = v.value
        for c in cands:
            assert L.pmg_tune_set(name.encode(), c) == 0
        assert L.pmg_tune_set(name.encode(), 0) == 0  # back to the default
        assert L.pmg_tune_get(name.encode(), ctypes.byref(v)) == 0 and v.value == default
    assert L.pmg_tune_set(b"cc.cross_fused", 1) == 0
    assert L.pmg_tune_set(b"cc.cross_fused", 0) == 0
    assert L.pmg_tune_get(b"cc.cross_fused", ctypes.byref(v)) == 0 and v.value == 0  # 0 is a value here
    assert L.pmg_tune_set(b"cc.cross_fused", 1) == 0
    assert L.pmg_tune_set(b"cc.cross_fused", -1) == 0
    assert L.pmg_tune_get(b"cc.cross_fused", ctypes.byref(v)) == 0 and v.value == 0
    assert L.pmg_tune_set(b"edt.pair_seg", 1) == _lib.PMG_ERANGE
    assert L.pmg_tune_set(b"no.such", 4) == _lib.PMG_EINVAL
    # path choices and probe thresholds: their defaults, 0 as a value, the
    # range ends, a negative value back to the default
    defaults = {b"edt.path": 0, b"edt.fallback": 96, b"edt.fallback_rows": 2048, b"edt.narrow": 64,
                b"edt.narrow_rows": 32, b"cc.seam_batched": 1, b"edt.wide": 1024}
    for name, default in defaults.items():
        assert L.pmg_tune_get(name, ctypes.byref(v)) == 0 and v.value == default
        assert L.pmg_tune_set(name, 0) == 0
        assert L.pmg_tune_get(name, ctypes.byref(v)) == 0 and v.value == 0
        assert L.pmg_tune_set(name, -1) == 0
        assert L.pmg_tune_get(name, ctypes.byref(v)) == 0 and v.value == default
    assert L.pmg_tune_set(b"edt.path", 3) == _lib.PMG_ERANGE
    assert L.pmg_tune_set(b"edt.fallback", 8193) == 0
    assert L.pmg_tune_set(b"edt.fallback", 8194) == _lib.PMG_ERANGE
    assert L.pmg_tune_set(b"edt.fallback", -1) == 0
    assert L.pmg_tune_set(b"cc.seam_batched", 2) == _lib.PMG_ERANGE
