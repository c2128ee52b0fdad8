"""Failure path of the bounded device loops (no GPU fault involved).

Every union-find root search and union retry stops at a bound and records a
status word instead of spinning; the entry point then returns PMG_EITER and
the Python layer raises PmgError (the reference raises or exits on a failed
distributed condition, src/pmmoto/core/utils.py:221-252).  The test lowers
the bounds to one iteration with the testing aid pmg_set_iteration_cap, so
the loops run out on ordinary inputs; it checks the error, then restores the
defaults and checks that the same CUDA context still gives correct results.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _geom(bts):
    from pmmoto_gb300.core import initialize

    vox = (62, 62, 62)
    box = tuple((0.0, v / 64) for v in vox)
    inlet = ((bts[0][0] == "end", False), (False, False), (False, False))
    outlet = ((False, bts[0][1] == "end"), (False, False), (False, False))
    sd = initialize(vox, box=box, boundary_types=bts, inlet=inlet, outlet=outlet)
    g = O.Geom(vox, boundary_types=bts, box=box, inlet=inlet, outlet=outlet)
    return sd, g


@pytest.mark.parametrize("bts,kind", [((("end", "end"),) * 3, "binary"),
                                      ((("periodic", "periodic"),) * 3, "binary"),
                                      ((("end", "end"), ("wall", "wall"), ("periodic", "periodic")), "multi")])
def test_iteration_cap_gives_error_then_context_works(bts, kind):
    from pmmoto_gb300 import _lib
    from pmmoto_gb300.filters import connected_components as C

    sd, g = _geom(bts)
    rng = np.random.default_rng(3)
    if kind == "binary":
        img = np.ones(sd.voxels, dtype=np.uint8)
        img[rng.random(sd.voxels) < 0.05] = 0
    else:
        img = np.where(rng.random(sd.voxels) < 0.5, 1, 2).astype(np.uint8)
    img = O.update_buffer(g, img)
    L = _lib.lib()
    assert L.pmg_set_iteration_cap(1) == 0
    try:
        with pytest.raises(_lib.PmgError, match="iteration cap"):
            C.connect_components(img, sd)
        if kind == "binary":
            with pytest.raises(_lib.PmgError, match="iteration cap"):
                C.inlet_connected_img(sd, img) if bts[0][0] == "end" else C.connect_components(img, sd)
    finally:
        assert L.pmg_set_iteration_cap(0) == 0
    lbl, n = C.connect_components(img, sd)
    want, wn = O.connect_components(img, g)
    np.testing.assert_array_equal(lbl, want)
    assert n == wn


def test_invalid_inputs_raise_value_errors():
    from pmmoto_gb300.filters import connected_components as C
    from pmmoto_gb300.filters import distance as D

    sd, _ = _geom((("end", "end"),) * 3)
    with pytest.raises(ValueError):
        D.edt(np.ones((4, 4), dtype=np.uint8).reshape(2, 2, 2, 2))
    with pytest.raises(ValueError):
        C.connect_components(np.ones((3, 3, 3), dtype=np.uint8), sd)
