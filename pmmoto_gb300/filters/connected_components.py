"""Drop-in for ``pmmoto.filters.connected_components`` on the GPU.

Same functions, arguments and return types as
src/pmmoto/filters/connected_components.py.  Labelling follows cc3d's
defaults as the reference calls it (26-connectivity, each nonzero value
separately, background 0, uint64 labels numbered by first voxel in C-order
scan); periodic seams are merged and renumbered as the reference does on one
rank.  The inlet/outlet selections depend only on the partition and run as
one fused union-find + face-mark + select pipeline.
"""

from __future__ import annotations

from collections import defaultdict

import numpy as np
import torch

from .. import _dev, tune
from .._lib import check, host_ptr, i64_array, lib
from ..core.geometry import geo_of

__all__ = ["connect_components", "gen_img_to_label_map", "phase_count", "inlet_outlet_labels",
           "inlet_outlet_connections", "inlet_connected_img", "outlet_connected_img",
           "inlet_outlet_connected_img", "isolated_img"]

SEL_INLET, SEL_OUTLET, SEL_BOTH, SEL_ISOLATED = 1, 2, 3, 4
SEL_BINARY = 16

_TORCH_BY_SIZE = {1: torch.uint8, 2: torch.int16, 4: torch.int32, 8: torch.int64}


def _img_device(img):
    """CUDA tensor of the image with its element size kept (values compared
    for equality only, so signedness does not matter)."""
    if isinstance(img, torch.Tensor):
        t, kind = _dev.to_device(img, img.dtype)
        if t.dtype == torch.bool:
            t = t.to(torch.uint8)
        if t.dtype.is_floating_point:
            t = t.to(torch.int64)
        return t.contiguous(), kind
    a = np.asarray(img)
    if a.dtype == np.bool_:
        a = a.view(np.uint8)
    if a.dtype.kind == "f":
        a = a.astype(np.int64)
    a = np.ascontiguousarray(a)
    view = a.view({1: np.uint8, 2: np.int16, 4: np.int32, 8: np.int64}[a.dtype.itemsize])
    t, _ = _dev.to_device(view, _TORCH_BY_SIZE[a.dtype.itemsize])
    return t, "numpy"


def connect_components_device(t: torch.Tensor, g):
    tune.apply("cc", t.shape)  # tuned launch parameters of this shape class, if any
    labels = torch.empty(t.shape, dtype=torch.int64, device=t.device)
    count = np.zeros(1, dtype=np.int64)
    st = lib().pmg_cc_label(_dev.ptr(t), t.element_size(), _dev.ptr(labels), host_ptr(i64_array(t.shape)),
                            host_ptr(g.bc_codes()), host_ptr(g.pad_flat()), host_ptr(count),
                            _dev.stream_ptr(t.device))
    check(st, "connect_components")
    return labels, int(count[0])


def connect_components(img, subdomain):
    """connected_components.py:32-62: (uint64 labels, label count)."""
    g = geo_of(subdomain)
    (t, kind) = _img_device(img)
    if tuple(t.shape) != g.shape:
        raise ValueError(f"image shape {tuple(t.shape)} != subdomain voxels {g.shape}")
    labels, count = connect_components_device(t, g)
    if kind == "torch":
        return labels, count
    return labels.cpu().numpy().view(np.uint64), count


def _box(slab):
    if slab is None:
        return np.full(6, -1, dtype=np.int64)
    return np.ascontiguousarray([v for lohi in slab for v in lohi], dtype=np.int64)


def select_device(g, t: torch.Tensor, mode: int, phase=None, out_dtype=torch.uint8):
    """Union-find with seams + face marks + selection, on a uint8 CUDA tensor."""
    if t.dtype != torch.uint8:
        raise ValueError("selection images must be uint8")
    out = torch.empty(t.shape, dtype=out_dtype, device=t.device)
    st = lib().pmg_cc_select(_dev.ptr(t), _dev.ptr(out), out.element_size(), host_ptr(i64_array(t.shape)),
                             host_ptr(g.bc_codes()), host_ptr(g.pad_flat()), host_ptr(_box(g.face_slab("inlet"))),
                             host_ptr(_box(g.face_slab("outlet"))), int(mode), -1 if phase is None else int(phase),
                             _dev.stream_ptr(t.device))
    check(st, "connected-image selection")
    return out


def _u8(img):
    from .morphological_operators import to_u8

    return to_u8(img)


def _select(subdomain, img, mode, phase):
    g = geo_of(subdomain)
    t, kind = _u8(img)
    if tuple(t.shape) != g.shape:
        raise ValueError(f"image shape {tuple(t.shape)} != subdomain voxels {g.shape}")
    out = select_device(g, t, mode, phase, torch.int64)
    if kind == "torch":
        return out
    return out.cpu().numpy().view(np.uint64)


def inlet_connected_img(subdomain, img, phase=None):
    """connected_components.py:254-296 (uint64 image of phase values)."""
    return _select(subdomain, img, SEL_INLET, phase)


def outlet_connected_img(subdomain, img, phase=None):
    """connected_components.py:299-341."""
    return _select(subdomain, img, SEL_OUTLET, phase)


def inlet_outlet_connected_img(subdomain, img, phase=None):
    """connected_components.py:203-251."""
    return _select(subdomain, img, SEL_BOTH, phase)


def isolated_img(subdomain, img, phase=None):
    """connected_components.py:344-392."""
    return _select(subdomain, img, SEL_ISOLATED, phase)


def gen_img_to_label_map(img, labeled_img):
    """connected_components.py:104-120: {label: phase}."""
    img_t, _ = _img_device(img)
    lab_t = labeled_img if isinstance(labeled_img, torch.Tensor) else torch.from_numpy(
        np.ascontiguousarray(np.asarray(labeled_img).view(np.int64))).cuda()
    lab_t = lab_t.to(img_t.device).view(torch.int64).reshape(-1)
    n = int(lab_t.max().item()) + 1 if lab_t.numel() else 1
    lut = torch.zeros(n, dtype=torch.int64, device=img_t.device)
    lut.scatter_(0, lab_t, img_t.reshape(-1).to(torch.int64))
    present = torch.zeros(n, dtype=torch.bool, device=img_t.device)
    present[lab_t] = True
    idx = torch.nonzero(present).flatten().cpu().numpy()
    vals = lut[present].cpu().numpy()
    return {np.uint64(k): np.uint64(v) for k, v in zip(idx, vals)}


def phase_count(phase_map):
    """connected_components.py:123-141."""
    out = {}
    for label in phase_map:
        out[phase_map[label]] = out.get(phase_map[label], 0) + 1
    return out


def inlet_outlet_labels(subdomain, labeled_img):
    """connected_components.py:144-177: {label: {"inlet": bool, "outlet": bool}}."""
    g = geo_of(subdomain)
    connected = defaultdict(lambda: {"inlet": False, "outlet": False})
    for which in ("inlet", "outlet"):
        slab = g.face_slab(which)
        if slab is None:
            continue
        face = labeled_img[tuple(slice(a, b) for a, b in slab)]
        face = face.cpu().numpy().view(np.uint64) if isinstance(face, torch.Tensor) else np.asarray(face)
        vals = np.unique(face)
        for label in vals:
            if label > 0:
                connected[np.uint64(label)][which] = True
    return connected


def inlet_outlet_connections(subdomain, labeled_img):
    """connected_components.py:180-200."""
    return [k for k, v in inlet_outlet_labels(subdomain, labeled_img).items() if v["inlet"] and v["outlet"]]
