"""Import the PMMoTo reference (installed under ``baseline/_ref``) in-process.

Test infrastructure only.  PMMoTo imports ``mpi4py``, ``matplotlib`` and the
third-party ``cc3d``; none is installed here, so small stand-ins are
registered first:

* ``mpi4py.MPI`` -- one rank: collectives return their input.
* ``matplotlib.pyplot`` -- inert (plotting is not on the path).
* ``cc3d.connected_components`` -- scipy.ndimage.label per nonzero value with
  the full 3x3x3 structure (26-connectivity, cc3d's default), renumbered
  1..N by first voxel in C-order raster scan (cc3d issues provisional labels
  in scan order and renumbers them consecutively).  Label *numbering* is an
  assumption because cc3d itself is absent; partitions and counts are not.

``load()`` returns the imported ``pmmoto`` module or None when the reference
install is missing (as on the GPU host).
"""

from __future__ import annotations

import os
import sys
import types

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF_SITE = os.path.join(REPO, "baseline", "_ref")


class _Op:
    def __init__(self, name):
        self.name = name


class _Comm:
    rank = 0
    size = 1

    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def allgather(self, x):
        return [x]

    def gather(self, x, root=0):
        return [x]

    def allreduce(self, x, op=None):
        return x

    def bcast(self, x, root=0):
        return x

    def Barrier(self):
        return None

    barrier = Barrier


def _install_stubs():
    if "mpi4py" not in sys.modules:
        mpi = types.ModuleType("mpi4py.MPI")
        mpi.COMM_WORLD = _Comm()
        mpi.Intracomm = _Comm
        mpi.Op = _Op
        for n in ("SUM", "PROD", "MAX", "MIN", "LAND", "BAND", "LOR", "BOR", "LXOR", "BXOR", "MINLOC", "MAXLOC"):
            setattr(mpi, n, _Op(n))

        class _Request:
            @staticmethod
            def waitall(reqs):
                return None

        mpi.Request = _Request
        pkg = types.ModuleType("mpi4py")
        pkg.MPI = mpi
        sys.modules["mpi4py"] = pkg
        sys.modules["mpi4py.MPI"] = mpi
    if "matplotlib" not in sys.modules:
        mpl = types.ModuleType("matplotlib")
        plt = types.ModuleType("matplotlib.pyplot")
        plt.__getattr__ = lambda name: (lambda *a, **k: None)  # type: ignore[attr-defined]
        mpl.pyplot = plt
        mpl.use = lambda *a, **k: None
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.pyplot"] = plt
    if "cc3d" not in sys.modules:
        cc = types.ModuleType("cc3d")
        cc.connected_components = cc3d_standin
        sys.modules["cc3d"] = cc


def cc3d_standin(data, return_N=False, out_dtype=None, connectivity=26, **_):
    from scipy import ndimage

    data = np.asarray(data)
    struct = ndimage.generate_binary_structure(data.ndim, data.ndim if connectivity == 26 else 1)
    first = []
    comp = np.zeros(data.shape, dtype=np.int64)
    offset = 0
    for v in np.unique(data):
        if v == 0:
            continue
        lab, n = ndimage.label(data == v, structure=struct)
        if n == 0:
            continue
        mask = lab > 0
        comp[mask] = lab[mask] + offset
        flat = lab.ravel()
        idx = np.flatnonzero(flat)
        _, firsts = np.unique(flat[idx], return_index=True)
        first.extend((idx[firsts]).tolist())
        offset += n
    order = np.argsort(np.asarray(first, dtype=np.int64), kind="stable")
    lut = np.zeros(offset + 1, dtype=np.uint64)
    lut[order + 1] = np.arange(1, offset + 1, dtype=np.uint64)
    out = lut[comp].astype(out_dtype or np.uint64)
    return (out, offset) if return_N else out


def load():
    if not os.path.isdir(os.path.join(REF_SITE, "pmmoto")):
        return None
    _install_stubs()
    if REF_SITE not in sys.path:
        sys.path.insert(0, REF_SITE)
    try:
        import pmmoto  # noqa: F401
    except Exception:  # pragma: no cover - x86 extension on another host
        return None
    return sys.modules["pmmoto"]
