"""The allocation-free EDT entry point, called through the C ABI.

pmg_edt3d_noalloc serves callers that cannot let the library allocate device
memory (a framework owning all device memory through its own pool, or a
latency-critical loop).  It must give exactly what pmg_edt3d gives -- the EDT
tests compare bit for bit, so the tolerance here is zero -- on consecutive
calls that reuse its fixed scratch arrays, must request no allocation at all
(the library's allocation counter stays put, while pmg_edt3d moves it), and
must refuse volumes beyond its 16,777,216 voxels.  The cases cover the
windowed envelope path (power-of-two voxels, lines of at most 1024 voxels),
the general path (a voxel size that is not a power of two) and a pass with
more lines than the fixed flag array holds (run in blocks of rows).

Collected last (file name) so a run that stops at the first failure has run
every other test before this one.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P = ctypes.c_void_p


def _lib():
    from pmmoto_gb300 import _lib as L

    lib = L.lib()
    for name in ("pmg_edt3d", "pmg_edt3d_noalloc"):
        fn = getattr(lib, name)
        fn.argtypes = [P, P, P, P, P, ctypes.c_int32, ctypes.c_int32, P]
        fn.restype = ctypes.c_int
    lib.pmg_scratch_alloc_count.restype = ctypes.c_longlong
    return lib, L


def _run(lib, L, name, img_t, periodic, res, form):
    import torch

    out = torch.full(tuple(img_t.shape), -1.0, dtype=torch.float32, device="cuda")
    shape = np.ascontiguousarray(img_t.shape, dtype=np.int64)
    resa = np.ascontiguousarray(res, dtype=np.float32)
    cfg = (L.AxisCfg * 3)(*[L.AxisCfg(int(p), 0, 0, 0, 1, 0, 0, 0) for p in periodic])
    stream = P(torch.cuda.current_stream().cuda_stream)
    st = getattr(lib, name)(P(img_t.data_ptr()), P(out.data_ptr()), P(shape.ctypes.data), P(resa.ctypes.data),
                            cfg, 4, form, stream)
    torch.cuda.synchronize()
    return st, out


def test_noalloc_matches_allocating_entry_point_twice():
    import torch

    lib, L = _lib()
    rng = np.random.default_rng(2026)
    cases = [((96, 80, 112), (True, True, True), (1.0, 1.0, 1.0), 0, 0.3),       # windowed path
             ((120, 64, 72), (False, True, False), (0.01, 0.01, 0.01), 1, 0.1),   # general path
             ((4096, 8, 512), (False, True, True), (0.5, 0.5, 0.5), 0, 0.2)]      # 2 Mi lines in pass 1
    for shape, periodic, res, form, p0 in cases:
        img = torch.as_tensor((rng.random(shape) >= p0).astype(np.uint8), device="cuda")
        a0 = lib.pmg_scratch_alloc_count()
        st_a, want = _run(lib, L, "pmg_edt3d", img, periodic, res, form)
        assert st_a == 0, L.last_error()
        assert lib.pmg_scratch_alloc_count() > a0  # the counter sees the allocating entry point
        for _ in range(2):  # two calls in a row share the fixed arrays
            a1 = lib.pmg_scratch_alloc_count()
            st_b, got = _run(lib, L, "pmg_edt3d_noalloc", img, periodic, res, form)
            assert st_b == 0, L.last_error()
            assert lib.pmg_scratch_alloc_count() == a1, "pmg_edt3d_noalloc requested an allocation"
            assert torch.equal(got, want)


def test_noalloc_rejects_volumes_beyond_its_scratch():
    import torch

    lib, L = _lib()
    img = torch.ones((257, 256, 256), dtype=torch.uint8, device="cuda")
    st, _ = _run(lib, L, "pmg_edt3d_noalloc", img, (False, False, False), (1.0, 1.0, 1.0), 0)
    assert st == L.PMG_ERANGE
    assert "exceeds the fixed scratch" in L.last_error()
