"""Device-memory helpers: accept numpy arrays or torch tensors, run on cuda:0
(or the tensor's device), and hand results back in the caller's container."""

from __future__ import annotations

import ctypes

import numpy as np
import torch


def require_cuda() -> None:
    if not torch.cuda.is_available():
        raise RuntimeError("pmmoto_gb300 needs a CUDA device (GB300, sm_103a); none is visible")


def to_device(a, dtype: torch.dtype):
    """Return (contiguous CUDA tensor of `dtype`, 'torch' | 'numpy')."""
    require_cuda()
    if isinstance(a, torch.Tensor):
        t = a if a.is_cuda else a.cuda()
        if t.dtype == torch.bool and dtype == torch.uint8:
            t = t.view(torch.uint8)
        return t.to(dtype).contiguous(), "torch"
    arr = np.asarray(a)
    if arr.dtype == np.bool_:
        arr = arr.view(np.uint8)
    t = torch.from_numpy(np.ascontiguousarray(arr))
    return t.to(device="cuda", dtype=dtype, non_blocking=False).contiguous(), "numpy"


def give_back(t: torch.Tensor, kind: str):
    return t if kind == "torch" else t.cpu().numpy()


class _DevPtr(ctypes.c_void_p):
    """A c_void_p holding a reference to the tensor it points into."""


def ptr(t: torch.Tensor) -> ctypes.c_void_p:
    if not t.is_cuda:
        raise ValueError("device pointers must come from CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("CUDA tensors passed to the C ABI must be contiguous")
    p = _DevPtr(t.data_ptr())
    p._keep = t
    return p


def stream_ptr(device=None) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
