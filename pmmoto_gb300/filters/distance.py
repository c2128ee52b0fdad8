"""Drop-in for ``pmmoto.filters.distance`` (EDT), computed on the GPU.

Same names, arguments, defaults and return dtypes as the reference
(src/pmmoto/filters/distance/euclidean_distance_transform.py): float32
distances (square-rooted unless ``squared=True``), bit-identical to the
reference on the same input.  Inputs may be numpy arrays (results come back
as numpy) or torch tensors (results stay on the device).
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _dev, tune
from .._lib import AxisCfg, EDT_DIST, EDT_SQUARED, check, i64_array, lib, host_ptr

__all__ = ["edt", "edt2d", "edt3d"]

NUM_HULL = 4  # euclidean_distance_transform.py:275,284


def _res32(resolution, nd):
    if len(resolution) != nd:
        raise ValueError(f"resolution must have {nd} entries")
    # the reference passes each resolution to a C `float` argument
    return np.ascontiguousarray([np.float32(r) for r in resolution], dtype=np.float32)


def edt3d_cfg(periodic):
    return (AxisCfg * 3)(*[AxisCfg(int(bool(p)), 0, 0, 0, 1, 0, 0, 0) for p in periodic])


def padded_cfg(pad, periodic_axes):
    """Axis rules of corrected_edt on a padded single-rank subdomain
    (euclidean_distance_transform.py:306-528): skips of 2*pad, correctors
    measured to the own region, the x+ face inheriting the x- lower skip."""
    cfg = []
    for d in range(3):
        lo, hi = int(pad[d][0]), int(pad[d][1])
        cfg.append(AxisCfg(int(bool(periodic_axes[d])), 2 * lo, 2 * lo, 2 * hi, -lo, -hi - 1, 2 * lo, 2 * hi))
    return (AxisCfg * 3)(*cfg)


def edt3d_device(t: torch.Tensor, res32: np.ndarray, cfg, squared: bool, out: torch.Tensor | None = None):
    """Squared (or plain) EDT of a contiguous uint8 CUDA tensor."""
    if t.dim() != 3:
        raise ValueError(f"Wrong img dimension {tuple(t.shape)}")
    if out is None:
        out = torch.empty(t.shape, dtype=torch.float32, device=t.device)
    tune.apply("edt", t.shape)  # tuned launch parameters of this shape class, if any
    shape = i64_array(t.shape)
    st = lib().pmg_edt3d(_dev.ptr(t), _dev.ptr(out), host_ptr(shape), host_ptr(res32), cfg, NUM_HULL,
                         EDT_SQUARED if squared else EDT_DIST, _dev.stream_ptr(t.device))
    check(st, "edt3d")
    return out


def edt3d(img, periodic=(False, False, False), resolution=(1.0, 1.0, 1.0), squared=False):
    """edt3d (euclidean_distance_transform.py:208-303)."""
    t, kind = _dev.to_device(img, torch.uint8)
    out = edt3d_device(t, _res32(resolution, 3), edt3d_cfg(periodic), squared)
    return _dev.give_back(out, kind)


def edt2d(img, periodic=(False, False), resolution=(1.0, 1.0)):
    """edt2d (euclidean_distance_transform.py:104-205)."""
    t, kind = _dev.to_device(img, torch.uint8)
    if t.dim() != 2:
        raise ValueError(f"Wrong img dimension {tuple(t.shape)}")
    out = torch.empty(t.shape, dtype=torch.float32, device=t.device)
    shape = i64_array(t.shape)
    per = np.ascontiguousarray([int(bool(p)) for p in periodic], dtype=np.int32)
    st = lib().pmg_edt2d(_dev.ptr(t), _dev.ptr(out), host_ptr(shape), host_ptr(_res32(resolution, 2)),
                         host_ptr(per), NUM_HULL, EDT_DIST, _dev.stream_ptr(t.device))
    check(st, "edt2d")
    return _dev.give_back(out, kind)


def _axis_periodic(subdomain):
    bts = subdomain.domain.boundary_types
    return [str(getattr(bts[d][0], "value", bts[d][0])) == "periodic" for d in range(3)]


def edt(img, subdomain=None):
    """edt (euclidean_distance_transform.py:25-53) for one rank on one GPU."""
    if subdomain is not None:
        if getattr(subdomain.domain, "num_subdomains", 1) > 1:
            raise NotImplementedError("pmmoto_gb300 runs one subdomain per GPU")
        res = subdomain.domain.resolution
        if subdomain.domain.periodic:
            t, kind = _dev.to_device(img, torch.uint8)
            out = edt3d_device(t, _res32(res, 3), padded_cfg(subdomain.pad, _axis_periodic(subdomain)), False)
            return _dev.give_back(out, kind)
        return edt3d(img, resolution=res)
    nd = img.dim() if isinstance(img, torch.Tensor) else np.ndim(img)
    if nd == 3:
        return edt3d(img)
    if nd == 2:
        return edt2d(img)
    raise ValueError(f"Wrong img dimension {tuple(np.shape(img))}")
