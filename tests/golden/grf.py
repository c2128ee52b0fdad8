"""Host twin of the device Gaussian-random-field generator
(``pmmoto_gb300.domain_generation.grf``), for the large-configuration
fixtures: ``grf_host.c`` (compiled here on first use) does the noise and the
smoothing with the same operations in the same order, numpy the threshold.
Test infrastructure; the package never imports it."""

from __future__ import annotations

import ctypes
import math
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
N_GRF = 1024
SEED = 7
POROSITY = 0.35
DESCRIPTION = ("hash noise U[-1/2,1/2) (lowbias32 twice of C index + seed*0x9E3779B9), periodic binomial B(64) "
               "smoothing per axis (sigma 4 voxels) in float64 without fused multiply-add, pore where field <= "
               "its k-th smallest value, k = round(0.35 N); seed 7")
_lib = None


def _load():
    global _lib
    if _lib is None:
        out = os.path.join(tempfile.gettempdir(), "pmg_grf_host.so")
        src = os.path.join(HERE, "grf_host.c")
        if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
            subprocess.run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                            "-fno-fast-math", src, "-o", out], check=True)
        L = ctypes.CDLL(out)
        P, i64 = ctypes.c_void_p, ctypes.c_int64
        L.grf_noise.argtypes = [P, i64, ctypes.c_uint32]
        L.grf_smooth_axis.argtypes = [P, P, i64, i64, i64, ctypes.c_int, P]
        _lib = L
    return _lib


def binomial_weights(order: int = 64) -> np.ndarray:
    return np.array([float(math.comb(order, k)) * 2.0 ** (-order) for k in range(order + 1)])


def grf_field_host(shape, seed: int = SEED) -> np.ndarray:
    L = _load()
    shape = tuple(int(s) for s in shape)
    a = np.empty(shape, dtype=np.float64)
    b = np.empty(shape, dtype=np.float64)
    L.grf_noise(a.ctypes.data, a.size, seed & 0xFFFFFFFF)
    w = np.ascontiguousarray(binomial_weights())
    for axis in range(3):
        L.grf_smooth_axis(a.ctypes.data, b.ctypes.data, *shape, axis, w.ctypes.data)
        a, b = b, a
    return a


def grf_medium_host(shape, porosity: float = POROSITY, seed: int = SEED) -> np.ndarray:
    if isinstance(shape, int):
        shape = (shape,) * 3
    f = grf_field_host(shape, seed)
    n = f.size
    k = max(1, min(n, int(round(porosity * n))))
    q = np.partition(f.reshape(-1).copy(), k - 1)[k - 1]
    return (f <= q).astype(np.uint8)
