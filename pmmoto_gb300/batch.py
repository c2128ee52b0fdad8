"""Many independent media on one GPU.

PMMoTo processes one subdomain per MPI rank; a batch of unrelated media
(sphere packs of different sizes, each with its own drainage sweep) has no
data exchange at all.  Small volumes leave most of a GB300 idle, so the batch
runs its media concurrently: a pool of host threads, each with its own CUDA
stream, takes media in turn and calls the ordinary single-medium entry
points on that stream (the C ABI takes the stream per call and allocates
scratch stream-ordered, and ctypes releases the GIL during each call).
Results are identical to running the media one after another.
"""

from __future__ import annotations

import threading
from concurrent.futures import ThreadPoolExecutor

import torch

__all__ = ["map_streams", "drainage_batch"]

_tls = threading.local()


def _thread_stream(device) -> torch.cuda.Stream:
    s = getattr(_tls, "stream", None)
    if s is None or s.device != torch.device(device):
        s = torch.cuda.Stream(device=device)
        _tls.stream = s
    return s


def map_streams(fn, items, workers: int = 8, device="cuda"):
    """[fn(item) for item in items], each call on one of `workers` CUDA
    streams of `device` (one per host thread); results in item order."""

    def run(item):
        s = _thread_stream(device)
        with torch.cuda.stream(s):
            out = fn(item)
        s.synchronize()
        return out

    if workers <= 1:
        return [run(it) for it in items]
    with ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(run, items))


def drainage_batch(multiphases, capillary_pressures, workers: int = 8, **kwargs):
    """equilibrium_distribution.drainage for every multiphase system of the
    list (each with its own capillary pressures, or one list for all);
    returns the list of saturation arrays."""
    from .filters.equilibrium_distribution import drainage

    if capillary_pressures and not hasattr(capillary_pressures[0], "__len__"):
        pcs = [capillary_pressures] * len(multiphases)
    else:
        pcs = list(capillary_pressures)
    if len(pcs) != len(multiphases):
        raise ValueError("one capillary-pressure list per multiphase system")
    return map_streams(lambda a: drainage(a[0], a[1], **kwargs), list(zip(multiphases, pcs)), workers)
