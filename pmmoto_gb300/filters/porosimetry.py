"""Drop-in for ``pmmoto.filters.porosimetry`` on the GPU
(src/pmmoto/filters/porosimetry.py:33-227).

Every mode of the reference is reproduced exactly: "distance" (EDT erosion and
dilation), "hybrid" (EDT erosion, FFT-ball dilation) and "morph" (FFT-ball
erosion and dilation) -- see morphological_operators for why the FFT ball is
an integer threshold of the same EDT.
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _dev
from .._lib import check, host_ptr, i64_array, lib
from ..core.geometry import geo_of
from . import morphological_operators as morph

__all__ = ["get_sizes", "porosimetry", "pore_size_distribution", "plot_pore_size_distribution"]

MODES = ("hybrid", "distance", "morph")


def get_sizes(min_value, max_value, num_values, spacing="linear"):
    """porosimetry.py:33-81."""
    if min_value >= max_value:
        raise ValueError(f"Error: min_value {min_value} must be greater than max value {max_value}")
    if num_values <= 0:
        raise ValueError(f"Error: num_values {num_values} must be greater than 0")
    if spacing == "linear":
        return np.linspace(min_value, max_value, num_values)[::-1]
    if spacing == "log":
        if min_value < 1:
            raise ValueError(f"Error: min_value {min_value} must be greater than or equal to 1")
        return np.logspace(np.log10(min_value), np.log10(max_value), num_values)[::-1]
    raise ValueError(f"spacing {spacing} can only be 'linear' or 'log'")


def _balls(g, r_e, r_d, mode):
    if mode not in MODES:
        raise ValueError(f"mode {mode} must be one of {MODES}")
    be = morph.ball_sq(g.res, r_e) if mode == "morph" else -1.0
    bd = morph.ball_sq(g.res, r_d) if mode in ("morph", "hybrid") else -1.0
    return be, bd


def porosimetry_device(g, pm: torch.Tensor, r_e, r_d, inlet: bool, mp: torch.Tensor | None, mode: str):
    ratio_e = np.ascontiguousarray(morph.element_ratio(g.res, r_e), dtype=np.int32)
    ratio_d = np.ascontiguousarray(morph.element_ratio(g.res, r_d), dtype=np.int32)
    be, bd = _balls(g, r_e, r_d, mode)
    out = torch.empty_like(pm)
    from .connected_components import _box

    res32 = np.ascontiguousarray([np.float32(r) for r in g.res], dtype=np.float32)
    st = lib().pmg_porosimetry(_dev.ptr(pm), _dev.ptr(mp) if mp is not None else None, _dev.ptr(out),
                               host_ptr(i64_array(pm.shape)), host_ptr(g.bc_codes()), host_ptr(g.pad_flat()),
                               host_ptr(_box(g.face_slab("inlet"))), host_ptr(res32), float(r_e),
                               int(morph.compare_in_float64(r_e)), host_ptr(ratio_e), float(r_d),
                               int(morph.compare_in_float64(r_d)), host_ptr(ratio_d), int(bool(inlet)), be, bd,
                               _dev.stream_ptr(pm.device))
    check(st, "porosimetry")
    return out


def porosimetry(subdomain, porous_media, radius, inlet=False, multiphase=None, mode="hybrid"):
    """porosimetry.py:84-160: erode, [inlet filter], [multiphase constraint], dilate."""
    if isinstance(radius, (int, float)):
        r_e = r_d = radius
    elif isinstance(radius, list) and len(radius) == 2:
        r_e, r_d = radius
    else:
        raise ValueError(f"Radius {radius} must either be a number or a list of length 2")
    morph.check_radii(subdomain, [r_e, r_d])
    g = geo_of(subdomain)
    pm, kind = morph.to_u8(porous_media.img)
    mp = None
    if multiphase is not None and hasattr(multiphase, "img"):
        mp, _ = morph.to_u8(multiphase.img)
    out = porosimetry_device(g, pm, r_e, r_d, inlet, mp, mode)
    return _dev.give_back(out, kind)


def pore_size_distribution(subdomain, porous_media, radii=None, num_radii=25, inlet=False, mode="hybrid"):
    """porosimetry.py:163-227: largest radius whose opening covers each pore voxel."""
    if radii is not None:
        if isinstance(radii, (int, float)):
            radii = [radii]
        elif isinstance(radii, list):
            radii.sort(reverse=True)
        elif isinstance(radii, np.ndarray):
            radii = np.sort(radii)[::-1]
    else:
        global_max = porous_media.max_distance
        rel_eps = 1e-6 * porous_media.max_distance
        global_max = global_max - rel_eps
        r_min = np.nextafter(np.min(subdomain.domain.resolution), np.inf)
        radii = get_sizes(r_min, global_max, num_radii, "linear")
    morph.check_radii(subdomain, radii)
    g = geo_of(subdomain)
    pm, kind = morph.to_u8(porous_media.img)
    out = torch.zeros(pm.shape, dtype=torch.float64, device=pm.device)
    pore = pm == 1
    for radius in radii:
        tmp = porosimetry_device(g, pm, radius, radius, inlet, None, mode)
        if bool(tmp.any()):
            sel = pore & (out == 0) & (tmp == 1)
            out = torch.where(sel, torch.as_tensor(float(radius), dtype=torch.float64, device=pm.device), out)
    return _dev.give_back(out, kind)


def plot_pore_size_distribution(*args, **kwargs):
    """Plotting is outside the GPU build (matplotlib is not a dependency)."""
    raise NotImplementedError("plotting is not part of pmmoto_gb300")
