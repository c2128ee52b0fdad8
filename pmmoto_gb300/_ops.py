"""Thin wrappers around the small device entry points (halo update,
reductions, sphere fill) shared by the drop-in modules."""

from __future__ import annotations

import numpy as np
import torch

from . import _dev
from ._lib import check, host_ptr, i64_array, lib


def box_all(shape):
    return np.ascontiguousarray([0, shape[0], 0, shape[1], 0, shape[2]], dtype=np.int64)


def box_of(slices_lohi):
    return np.ascontiguousarray([v for lohi in slices_lohi for v in lohi], dtype=np.int64)


def update_buffer_device(t: torch.Tensor, g) -> torch.Tensor:
    st = lib().pmg_update_buffer(_dev.ptr(t), t.element_size(), host_ptr(i64_array(t.shape)),
                                 host_ptr(g.bc_codes()), host_ptr(g.pad_flat()), _dev.stream_ptr(t.device))
    check(st, "update_buffer")
    return t


def count_eq_device(t: torch.Tensor, box, value: int) -> int:
    out = np.zeros(1, dtype=np.int64)
    st = lib().pmg_count_eq(_dev.ptr(t), host_ptr(i64_array(t.shape)), host_ptr(np.ascontiguousarray(box, np.int64)),
                            int(value), host_ptr(out), _dev.stream_ptr(t.device))
    check(st, "count")
    return int(out[0])


def max_f32_device(t: torch.Tensor, box=None) -> float:
    out = np.zeros(1, dtype=np.float32)
    box = box_all(t.shape) if box is None else np.ascontiguousarray(box, np.int64)
    st = lib().pmg_max_f32(_dev.ptr(t), host_ptr(i64_array(t.shape)), host_ptr(box), host_ptr(out),
                           _dev.stream_ptr(t.device))
    check(st, "max")
    return float(out[0])


def spheres_device(spheres, coords, device="cuda") -> torch.Tensor:
    """Sphere fill of a padded grid whose voxel centres are `coords`."""
    if isinstance(spheres, torch.Tensor):
        sph = spheres.to(device=device, dtype=torch.float64).reshape(-1, 4).contiguous()
    else:
        sph = torch.as_tensor(np.ascontiguousarray(np.asarray(spheres, dtype=np.float64).reshape(-1, 4)),
                              device=device)
    cs = [torch.as_tensor(np.ascontiguousarray(c, dtype=np.float64), device=device) for c in coords]
    shape = tuple(int(c.shape[0]) for c in cs)
    img = torch.empty(shape, dtype=torch.uint8, device=device)
    c0 = np.ascontiguousarray([float(c[0]) for c in coords], dtype=np.float64)
    h = np.ascontiguousarray([float(c[1] - c[0]) if len(c) > 1 else 1.0 for c in coords], dtype=np.float64)
    st = lib().pmg_spheres(_dev.ptr(sph), int(sph.shape[0]), _dev.ptr(cs[0]), _dev.ptr(cs[1]), _dev.ptr(cs[2]),
                           host_ptr(c0), host_ptr(h), _dev.ptr(img), host_ptr(i64_array(shape)),
                           _dev.stream_ptr(img.device))
    check(st, "sphere voxelisation")
    return img
