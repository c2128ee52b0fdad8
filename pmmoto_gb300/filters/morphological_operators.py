"""Drop-in for ``pmmoto.filters.morphological_operators`` on the GPU.

Same functions and arguments as src/pmmoto/filters/morphological_operators.py.
Both variants run as one CUDA pipeline (wrap extension of the periodic faces,
exact EDT, threshold, unpad and wall rule fused):

* ``fft=False`` -- the reference's EDT path: ``sqrt(d2) <= radius`` in the
  precision numpy uses for the comparison.
* ``fft=True`` -- the reference convolves with the structuring element
  ``{(i, j, k) : i*i + j*j + k*k <= (radius/res)**2}`` (scipy fftconvolve,
  thresholded at 0.1 / sum - 0.1).  A voxel is reached by a 1-voxel through
  that element exactly when the squared voxel-unit distance to the nearest
  1-voxel is at most ``floor((radius/res)**2)``, so the same EDT kernels with
  unit resolution and that integer bound give the convolution's result.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from .. import _dev
from .._lib import check, host_ptr, i64_array, lib
from ..core.geometry import geo_of

__all__ = ["gen_struct_ratio", "gen_struct_element", "addition", "dilate", "subtraction", "erode",
           "opening", "closing", "check_radii"]


def gen_struct_ratio(resolution, radius):
    """morphological_operators.py:35-63."""
    if len(resolution) not in {2, 3}:
        raise ValueError("Resolution must be a list of length 2 or 3")
    if radius < np.min(resolution):
        raise ValueError(f"The chosen radius {radius} is too small! The resolutions is {resolution}")
    return tuple(int(math.ceil(radius / res)) for res in resolution)


def gen_struct_element(resolution, radius):
    """morphological_operators.py:66-100 (the element itself is host-side)."""
    if len(resolution) not in {2, 3}:
        raise ValueError("Resolution must be a list or tuple of length 2 or 3.")
    if resolution[0] != resolution[1] != resolution[2]:
        raise ValueError("Resolution must be isotropic for morphological methods.")
    ratio = gen_struct_ratio(resolution, radius)
    grids = [np.linspace(-r, r, r * 2 + 1) for r in ratio]
    xg, yg, zg = np.meshgrid(*grids, indexing="ij")
    s = xg**2 + yg**2 + zg**2
    r = radius / resolution[0]
    return ratio, np.array(s <= r * r, dtype=np.uint8)


def element_ratio(resolution, radius):
    """gen_struct_element's checks and ratio without building the element
    (the device paths only need the ratio)."""
    if len(resolution) not in {2, 3}:
        raise ValueError("Resolution must be a list or tuple of length 2 or 3.")
    if resolution[0] != resolution[1] != resolution[2]:
        raise ValueError("Resolution must be isotropic for morphological methods.")
    return gen_struct_ratio(resolution, radius)


def compare_in_float64(radius) -> bool:
    """The dtype numpy uses for ``float32_array <= radius`` (NEP 50): Python
    scalars are weak (float32 compare); numpy scalars promote normally."""
    if isinstance(radius, (np.generic, np.ndarray)):
        return np.result_type(np.float32, np.asarray(radius).dtype) != np.float32
    return False


def _check_buffer(g, ratio):
    """check_subdomain_condition in update_extended_buffer (communication.py:140-150):
    the reference logs the error and exits the process."""
    if any(g.own_voxels[d] < ratio[d] for d in range(3)):
        raise SystemExit(1)


def _ext(g, ratio):
    """extend_padding (subdomain_padded.py:116-167) on one rank."""
    ext = []
    for d in range(3):
        for s in (0, 1):
            b = g.bts[d][s]
            ext.append(0 if b == "end" or (b == "wall" and g.pad[d][s] == 1) else int(ratio[d]))
    return np.ascontiguousarray(ext, dtype=np.int32)


def to_u8(img):
    """uint8 CUDA tensor of an image whose values lie in [0, 255]."""
    if not isinstance(img, torch.Tensor):
        a = np.asarray(img)
        if a.dtype not in (np.uint8, np.bool_) and a.size and (a.max() > 255 or a.min() < 0):
            raise ValueError("morphology input values must lie in [0, 255]")
        return _dev.to_device(a.astype(np.uint8, copy=False), torch.uint8)
    t, kind = _dev.to_device(img, img.dtype)
    if t.dtype != torch.uint8:
        if t.dtype.is_floating_point or t.dtype == torch.bool or t.numel() == 0:
            t = t.to(torch.uint8)
        else:
            if bool((t > 255).any()) or bool((t < 0).any()):
                raise ValueError("morphology input values must lie in [0, 255]")
            t = t.to(torch.uint8)
    return t.contiguous(), kind


def ball_sq(resolution, radius) -> float:
    """floor of (radius/res)^2 as gen_struct_element forms it (float64)."""
    r = radius / resolution[0]
    return float(np.floor(r * r))


def morph_device(g, t: torch.Tensor, radius, dilate: bool, out: torch.Tensor | None = None, fft: bool = False):
    """Addition/subtraction of a contiguous uint8 CUDA tensor of the padded shape."""
    ratio = element_ratio(g.res, radius)
    _check_buffer(g, ratio)
    if tuple(t.shape) != g.shape:
        raise ValueError(f"image shape {tuple(t.shape)} != subdomain voxels {g.shape}")
    if out is None:
        out = torch.empty_like(t)
    res32 = np.ascontiguousarray([np.float32(r) for r in g.res], dtype=np.float32)
    st = lib().pmg_morph(_dev.ptr(t), _dev.ptr(out), host_ptr(i64_array(g.shape)), host_ptr(g.bc_codes()),
                         host_ptr(g.pad_flat()), host_ptr(_ext(g, ratio)), host_ptr(res32), float(radius),
                         int(compare_in_float64(radius)), int(bool(dilate)),
                         ball_sq(g.res, radius) if fft else -1.0, _dev.stream_ptr(t.device))
    check(st, "addition" if dilate else "subtraction")
    return out


def _run(subdomain, img, radius, fft, dilate):
    g = geo_of(subdomain)
    t, kind = to_u8(img)
    return _dev.give_back(morph_device(g, t, radius, dilate, fft=bool(fft)), kind)


def addition(subdomain, img, radius, fft=False):
    """Morphological dilation (morphological_operators.py:103-149)."""
    return _run(subdomain, img, radius, fft, True)


def dilate(subdomain, img, radius, fft=False):
    return addition(subdomain, img, radius, fft)


def subtraction(subdomain, img, radius, fft=False):
    """Morphological erosion (morphological_operators.py:175-228)."""
    return _run(subdomain, img, radius, fft, False)


def erode(subdomain, img, radius, fft=False):
    return subtraction(subdomain, img, radius, fft)


def opening(subdomain, img, radius, fft=False):
    """Erosion followed by dilation (morphological_operators.py:254-274)."""
    return addition(subdomain, subtraction(subdomain, img, radius, fft), radius, fft)


def closing(subdomain, img, radius, fft=False):
    """Dilation followed by erosion (morphological_operators.py:277-297)."""
    return subtraction(subdomain, addition(subdomain, img, radius, fft), radius, fft)


def check_radii(subdomain, radii):
    """morphological_operators.py:300-329."""
    g = geo_of(subdomain)
    for radius in radii:
        ratio = element_ratio(g.res, radius)
        _check_buffer(g, ratio)
