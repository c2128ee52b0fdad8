"""Gaussian random field media on the device (a new generator: the
reference's ``gen_img_smoothed_random_binary``, domain_generation.py:63-100,
is a different model).

The medium of the large EDT + connected-components configuration and of the
learned radius schedule's training set: white noise, smoothed by a periodic
Gaussian of sigma = 4 voxels per axis, pore (1) where the field is at or below
its q-quantile (q = the porosity), solid (0) elsewhere.

Every operation is reproducible bit for bit on any IEEE-754 machine, so a
host generator and the device produce the same bytes (a digest of the medium
pins both sides to the same input):

* noise: a 32-bit integer hash (lowbias32, applied twice) of the voxel's C
  index plus a seed offset, mapped to u = h * 2^-32 - 1/2 (exact in float64);
* smoothing: along each axis in turn (0, 1, 2), a periodic convolution with
  the 65-tap binomial kernel w_k = C(64, k) / 2^64 (variance 64/4 = 16 =
  sigma^2; the binomial kernel approaches the Gaussian), evaluated in float64
  as acc = w_0 x_{i-32}, then acc = acc + w_k x_{i+k-32} for k = 1..64, each
  product and sum rounded once (separate multiply and add kernels, no fused
  multiply-add) -- the filtering a Fourier-space Gaussian does, in an operation
  order that does not depend on an FFT library;
* threshold: q = the k-th smallest field value, k = round(porosity * N);
  pore where field <= q.
"""

from __future__ import annotations

import math

import numpy as np
import torch

SIGMA_TAPS = 64  # binomial order: variance SIGMA_TAPS / 4 = 16 (sigma 4 voxels)
HALF = SIGMA_TAPS // 2
_M32 = 0xFFFFFFFF


def binomial_weights(order: int = SIGMA_TAPS) -> list[float]:
    """w_k = C(order, k) / 2^order as float64 (int -> float correctly rounded,
    the power-of-two scaling exact)."""
    return [float(math.comb(order, k)) * 2.0 ** (-order) for k in range(order + 1)]


def _mul32(x: torch.Tensor, c: int) -> torch.Tensor:
    """(x * c) mod 2^32 for int64 tensors holding values in [0, 2^32), without
    int64 overflow (the constant is split in 16-bit halves)."""
    lo, hi = c & 0xFFFF, c >> 16
    return (x * lo + (((x * hi) & 0xFFFF) << 16)) & _M32


def _lowbias32(x: torch.Tensor) -> torch.Tensor:
    x = x ^ (x >> 16)
    x = _mul32(x, 0x7FEB352D)
    x = x ^ (x >> 15)
    x = _mul32(x, 0x846CA68B)
    return x ^ (x >> 16)


def noise(shape, seed: int, device="cuda") -> torch.Tensor:
    """Uniform white noise in [-1/2, 1/2) (float64) from the hashed C index."""
    n = int(math.prod(shape))
    off = (int(seed) * 0x9E3779B9) & _M32
    x = (torch.arange(n, dtype=torch.int64, device=device) + off) & _M32
    h = _lowbias32(_lowbias32(x))
    del x
    return (h.to(torch.float64) * 2.0 ** -32 - 0.5).reshape(tuple(shape))


def smooth(field: torch.Tensor, dims=None, order: int = SIGMA_TAPS) -> torch.Tensor:
    """Periodic binomial smoothing along each of `dims` (default: the last
    three) in the fixed operation order of the module docstring; `order` is
    the binomial order (even; sigma = sqrt(order) / 2 voxels)."""
    w = binomial_weights(order)
    half = order // 2
    dims = tuple(range(field.dim() - 3, field.dim())) if dims is None else dims
    x = field
    for d in dims:
        acc = torch.mul(torch.roll(x, half, d), w[0])
        for k in range(1, order + 1):
            acc = torch.add(acc, torch.mul(torch.roll(x, half - k, d), w[k]))
        x = acc
    return x


def smooth_device(field: torch.Tensor, order: int = SIGMA_TAPS) -> torch.Tensor:
    """smooth() over the last three axes of a CUDA float64 tensor with the
    library's smoothing kernel (one pass per axis, the same operations in the
    same order, so the same bytes as smooth())."""
    import ctypes

    from .._lib import check, host_ptr, i64_array, lib

    L = lib()
    src = field.contiguous()
    shape = src.shape[-3:]
    batch = int(math.prod(src.shape[:-3])) if src.dim() > 3 else 1
    w = np.ascontiguousarray(binomial_weights(order), dtype=np.float64)
    a, b = torch.empty_like(src), torch.empty_like(src)  # the input is never written
    st = ctypes.c_void_p(torch.cuda.current_stream(src.device).cuda_stream)
    for axis, (x, y) in enumerate(((src, a), (a, b), (b, a))):
        check(L.pmg_grf_smooth(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), batch,
                               host_ptr(i64_array(shape)), axis, host_ptr(w), order, st), "grf smooth")
    del b
    return a


def order_for_sigma(sigma: float) -> int:
    """Even binomial order whose variance order / 4 is closest to sigma^2."""
    return max(2, 2 * int(round(2.0 * sigma * sigma)))


def grf_field(shape, seed: int = 7, device="cuda", sigma: float = 4.0) -> torch.Tensor:
    """The smoothed field (float64) of one medium (the library kernel on a
    CUDA device, the tensor formulation elsewhere: the same bytes)."""
    f = noise(shape, seed, device)
    if f.is_cuda:
        return smooth_device(f, order_for_sigma(sigma))
    return smooth(f, order=order_for_sigma(sigma))


def threshold(f: torch.Tensor, porosity) -> torch.Tensor:
    """Pore (1) where each medium's field is at or below its k-th smallest
    value, k = round(porosity * N); f: [..., n0, n1, n2]."""
    lead = f.shape[:-3]
    flat = f.reshape(-1, int(math.prod(f.shape[-3:])))
    por = np.broadcast_to(np.asarray(porosity, dtype=np.float64), (flat.shape[0],))
    n = flat.shape[1]
    q = torch.empty(flat.shape[0], dtype=f.dtype, device=f.device)
    if n <= (1 << 26):
        srt = torch.sort(flat, dim=1).values
        for i in range(flat.shape[0]):
            q[i] = srt[i, max(1, min(n, int(round(float(por[i]) * n)))) - 1]
        del srt
    else:
        for i in range(flat.shape[0]):
            q[i] = torch.kthvalue(flat[i], max(1, min(n, int(round(float(por[i]) * n))))).values
    return (f <= q.view(*lead, 1, 1, 1) if lead else f <= q[0]).to(torch.uint8)


def gen_grf_medium(shape, porosity: float = 0.35, seed: int = 7, device="cuda", sigma: float = 4.0) -> torch.Tensor:
    """uint8 medium of `shape` (1 = pore where the field is at or below its
    porosity-quantile) on `device`; sigma in voxels (4: the large EDT + CC
    configuration)."""
    if isinstance(shape, int):
        shape = (shape,) * 3
    return threshold(grf_field(shape, seed, device, sigma), porosity)
