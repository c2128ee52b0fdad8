"""Loader for the CUDA library (``_lib/libpmmoto_gb300.so``) and call helpers.

The library is the only compute path: if it is missing or no CUDA device is
visible, every operator raises instead of falling back to the CPU.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

_lock = threading.Lock()
_lib = None

PMG_OK = 0
PMG_EINVAL = 1
PMG_ERANGE = 2
PMG_ECUDA = -1
PMG_EITER = -2

BC_END, BC_WALL, BC_PERIODIC = 0, 1, 2
EDT_SQUARED, EDT_DIST = 0, 1


class AxisCfg(ctypes.Structure):
    """``pmg_axis_cfg`` of include/pmmoto_gb300.h."""

    _fields_ = [(n, ctypes.c_int32) for n in ("periodic", "f_lo", "l_lo", "l_hi", "a_u", "a_l", "hf_lo", "hb_hi")]


class PmgError(RuntimeError):
    """A failure reported by the CUDA library."""


def _declare(L):
    P = ctypes.c_void_p
    i32, i64 = ctypes.c_int32, ctypes.c_int64
    f64 = ctypes.c_double
    sig = {
        "pmg_edt3d": [P, P, P, P, P, i32, i32, P],
        "pmg_edt2d": [P, P, P, P, P, i32, i32, P],
        "pmg_morph": [P, P, P, P, P, P, P, f64, i32, i32, f64, P],
        "pmg_cc_label": [P, i32, P, P, P, P, P, P],
        "pmg_cc_select": [P, P, i32, P, P, P, P, P, i32, i32, P],
        "pmg_spheres": [P, i64, P, P, P, P, P, P, P, P],
        "pmg_update_buffer": [P, i32, P, P, P, P],
        "pmg_count_eq": [P, P, P, i32, P, P],
        "pmg_max_f32": [P, P, P, P, P],
        "pmg_porosimetry": [P, P, P, P, P, P, P, P, f64, i32, P, f64, i32, P, i32, f64, f64, P],
        "pmg_drainage": [P, P, P, P, P, P, P, P, P, P, i32, P, P, P, P, P, P, P],
        "pmg_drainage_ext": [P, P, P, P, P, P, P, P, P, P, i32, P, P, P, P, P, P, P, P, P],
        "pmg_last_error": [ctypes.c_char_p, ctypes.c_size_t],
        "pmg_set_iteration_cap": [i32],
        "pmg_grf_smooth": [P, P, i64, P, i32, P, i32, P],
        "pmg_tune_set": [ctypes.c_char_p, i32],
        "pmg_tune_get": [ctypes.c_char_p, P],
    }
    for name, args in sig.items():
        if hasattr(L, name):
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
    L.pmg_version.restype = ctypes.c_char_p
    L.pmg_launch_count.restype = ctypes.c_longlong
    L.pmg_scratch_alloc_count.restype = ctypes.c_longlong


def lib():
    """Return the loaded library; build it in-tree when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not os.path.exists(path):
                _build.build()
            L = ctypes.CDLL(path)
            _declare(L)
            _lib = L
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    lib().pmg_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status: int, what: str) -> None:
    if status == PMG_OK:
        return
    msg = last_error()
    if status in (PMG_EINVAL, PMG_ERANGE):
        raise ValueError(f"{what}: {msg}")
    raise PmgError(f"{what} failed (status {status}): {msg}")


def i64_array(vals) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(vals, dtype=np.int64))


class _HostPtr(ctypes.c_void_p):
    """A c_void_p that owns a reference to the array it points into, so an
    array built inline in an argument list lives until the call returns."""


def host_ptr(a: np.ndarray) -> ctypes.c_void_p:
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("host arrays passed to the C ABI must be C-contiguous")
    p = _HostPtr(a.ctypes.data)
    p._keep = a
    return p
