"""Autotuner of launch parameters (no counterpart in the reference).

Some launch parameters change only speed, never results: the line-pair
envelope passes' segment length and CTA counts (library knobs set through
``pmg_tune_set``) and the number of CUDA streams the batched configuration
spreads its media over (a host-side knob).  The tuner times every candidate
of one knob at a time (coordinate descent, the others held at their current
best) on a synthetic medium of the caller's shape class, with CUDA events
after a warm-up, and keeps the fastest.

Results are cached as JSON (``$PMG_TUNE_CACHE``, default
``~/.cache/pmmoto_gb300/autotune.json``) under the key
``<GPU name>|<kernel>|<shape class>``, where the shape class rounds every
extent up to a power of two.  ``apply`` looks the key up once per process
and sets the library knobs; ``PMG_TUNE="name=value,..."`` overrides cached
values (used by tests and to pin a configuration).
"""

from __future__ import annotations

import json
import math
import os
import threading

import numpy as np

KNOBS = {
    "edt": {"edt.pair_seg": [128, 256, 512, 1024], "edt.pair_ctas": [8, 16, 32, 64],
            "edt.rows_ctas": [4, 8, 16, 32]},
    "cc": {"cc.cross_fused": [0, 1]},
    "batch": {"batch.workers": [2, 4, 8, 16]},
}
HOST_KNOBS = {"batch.workers": 8}
_lock = threading.Lock()
_applied: dict[str, dict] = {}


def cache_path() -> str:
    return os.environ.get("PMG_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "pmmoto_gb300", "autotune.json"))


def shape_class(shape) -> str:
    return "x".join(str(1 << max(0, math.ceil(math.log2(max(1, int(s)))))) for s in shape)


def gpu_name() -> str:
    import torch

    return torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"


def key(kernel: str, shape, gpu: str | None = None) -> str:
    return f"{gpu or gpu_name()}|{kernel}|{shape_class(shape)}"


def overrides() -> dict:
    """PMG_TUNE="name=value,..." as {name: int}."""
    out = {}
    for part in os.environ.get("PMG_TUNE", "").split(","):
        part = part.strip()
        if not part:
            continue
        name, _, val = part.partition("=")
        if not val:
            raise ValueError(f"PMG_TUNE entry {part!r} is not name=value")
        out[name.strip()] = int(val)
    return out


def load_cache() -> dict:
    p = cache_path()
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f)


def save_entry(k: str, settings: dict, timings: dict) -> None:
    with _lock:
        d = load_cache()
        d[k] = {"settings": settings, "ms": timings}
        p = cache_path()
        os.makedirs(os.path.dirname(p) or ".", exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)


def _set_lib(name: str, value: int) -> None:
    from ._lib import check, lib

    check(lib().pmg_tune_set(name.encode(), int(value)), "tune")


def reset_lib(kernel: str) -> None:
    """Defaults for every library knob of `kernel`."""
    for name in KNOBS.get(kernel, {}):
        if name not in HOST_KNOBS:
            _set_lib(name, -1)


def get_lib(name: str) -> int:
    import ctypes

    from ._lib import check, lib

    v = ctypes.c_int32(0)
    check(lib().pmg_tune_get(name.encode(), ctypes.byref(v)), "tune")
    return int(v.value)


def settings_for(kernel: str, shape) -> dict:
    """Cached settings of (kernel, shape class) on this GPU, overridden by
    PMG_TUNE; {} when nothing is known."""
    s = dict(load_cache().get(key(kernel, shape), {}).get("settings", {}))
    ov = overrides()
    for name in KNOBS.get(kernel, {}):
        if name in ov:
            s[name] = ov[name]
    return s


def apply(kernel: str, shape) -> dict:
    """Set the library knobs of `kernel` for this shape class (once per
    process and class); returns the settings in force."""
    k = key(kernel, shape)
    if k not in _applied:
        s = settings_for(kernel, shape)
        for name, v in s.items():
            if name not in HOST_KNOBS:
                _set_lib(name, v)
        _applied[k] = s
    return _applied[k]


def host_value(kernel: str, shape, name: str) -> int:
    return int(settings_for(kernel, shape).get(name, HOST_KNOBS[name]))


def _time(fn, steps: int) -> float:
    import torch

    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _descend(kernel: str, shape, run, steps: int, set_knob) -> tuple[dict, dict]:
    best, timings = {}, {}
    for name, cands in KNOBS[kernel].items():
        res = {}
        for c in cands:
            set_knob(name, c)
            res[c] = _time(run, steps)
        pick = min(res, key=res.get)
        set_knob(name, pick)
        best[name] = pick
        timings[name] = {str(c): round(t, 4) for c, t in res.items()}
    return best, timings


def tune_edt(shape, periodic=(True, True, True), steps: int = 3, force: bool = False) -> dict:
    """Tune the EDT's line-pair passes for `shape` on a GRF medium of that
    shape (porosity 0.35, sigma 4 voxels); cached per shape class."""
    import torch

    from .domain_generation import grf
    from .filters import distance as D

    k = key("edt", shape)
    if not force:
        cached = load_cache().get(k)
        if cached:
            _applied.pop(k, None)
            return apply("edt", shape)
    img = grf.gen_grf_medium(tuple(int(s) for s in shape))
    out = torch.empty(img.shape, dtype=torch.float32, device=img.device)
    cfg = D.edt3d_cfg(periodic)
    res = np.ones(3, np.float32)
    best, timings = _descend("edt", shape, lambda: D.edt3d_device(img, res, cfg, True, out), steps, _set_lib)
    save_entry(k, best, timings)
    _applied[k] = best
    return best


def tune_cc(shape, steps: int = 3, force: bool = False) -> dict:
    """Tune the block labelling for padded periodic volumes of `shape` on a GRF
    medium (porosity 0.35, sigma 4 voxels); cached per shape class."""
    import pmmoto_gb300 as P

    from .core.geometry import geo_of
    from .domain_generation import grf
    from .filters import connected_components as CC

    k = key("cc", shape)
    if not force and load_cache().get(k):
        _applied.pop(k, None)
        return apply("cc", shape)
    own = grf.gen_grf_medium(tuple(int(s) - 2 for s in shape))
    import torch

    idx = [torch.arange(-1, n + 1, device=own.device) % n for n in own.shape]
    img = own[idx[0]][:, idx[1]][:, :, idx[2]].contiguous()
    sd = P.initialize(tuple(own.shape), boundary_types=(("periodic", "periodic"),) * 3)
    geo = geo_of(sd)
    best, timings = _descend("cc", shape, lambda: CC.connect_components_device(img, geo), steps, _set_lib)
    save_entry(k, best, timings)
    _applied[k] = best
    return best


def tune_batch(items, fn, steps: int = 1, force: bool = False) -> dict:
    """Tune the number of CUDA streams of batch.map_streams(fn, items) for the
    shape class of the batch's largest medium (items: (voxels, ...) tuples)."""
    from . import batch

    shape = tuple(max(int(it[0][d]) for it in items) for d in range(3))
    k = key("batch", shape)
    if not force and k in load_cache():
        return settings_for("batch", shape)
    cur = {}

    def run():
        batch.map_streams(fn, items, workers=cur["batch.workers"])

    best, timings = _descend("batch", shape, run, steps, lambda n, v: cur.__setitem__(n, v))
    save_entry(k, best, timings)
    return best
