"""Pin the oracle (CPU restatement) to the reference.

* against the golden fixtures generated from PMMoTo itself
  (tests/golden/make_golden.py) -- runs everywhere;
* against PMMoTo's own C++ line kernels compiled from its sources
  (oracle/_ref/libpmref.so) on random lines -- runs where those sources were
  available to build the library.
"""

import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle import build as OB
from tests._helpers import geom_from_meta


def test_kat_pass0(golden):
    np.testing.assert_array_equal(O.initial_envelope_1d(golden["kat_pass0_in"]), golden["kat_pass0_out"])
    np.testing.assert_array_equal(O.initial_envelope_1d(golden["kat_pass0c_in"], 1, 1), golden["kat_pass0c_out_11"])
    np.testing.assert_array_equal(O.initial_envelope_1d(golden["kat_pass0c_in"], 2, 4), golden["kat_pass0c_out_24"])


def test_kat_boundary_hull(golden, golden_meta):
    hin = golden["kat_hull_in"]
    for (s, e, nh, fwd), want in zip(golden_meta["kat_hulls"]["cases"], golden_meta["kat_hulls"]["hulls"]):
        got = O.boundary_hull_1d(np.r_[hin, np.float32(np.inf)], s, e, 1.0, nh, fwd)
        got = [[h["vertex"], h["height"], h["range"]] for h in got]
        assert got == want


@pytest.mark.parametrize("ci", range(6))
def test_edt3d_golden(golden, golden_meta, ci):
    c = golden_meta["edt3d_cases"][ci]
    out = O.edt3d(golden[f"edt3d_{ci}_in"], periodic=c["periodic"], resolution=c["resolution"], squared=True)
    np.testing.assert_array_equal(out, golden[f"edt3d_{ci}_out"])


def test_edt3d_labels_golden(golden):
    np.testing.assert_array_equal(O.edt3d(golden["edt3d_labels_in"], squared=True), golden["edt3d_labels_out"])


def test_edt2d_golden(golden):
    np.testing.assert_array_equal(O.edt2d(golden["edt2d_in"], periodic=(True, True)), golden["edt2d_out_p"])
    np.testing.assert_array_equal(O.edt2d(golden["edt2d_in"]), golden["edt2d_out_n"])


@pytest.mark.parametrize("ci", range(5))
def test_subdomain_golden(golden, golden_meta, ci):
    case = golden_meta["sub_cases"][ci]
    g = geom_from_meta(O, case["geom"])
    img = O.gen_pm_spheres_domain(g, golden[f"sub_{ci}_spheres"])
    np.testing.assert_array_equal(img, golden[f"sub_{ci}_img"])
    np.testing.assert_array_equal(O.edt(img, g), golden[f"sub_{ci}_edt"])
    lbl, n = O.connect_components(img, g)
    np.testing.assert_array_equal(lbl, golden[f"sub_{ci}_cc"])
    assert n == case["cc_count"]
    for ri, r in enumerate(case["radii"]):
        np.testing.assert_array_equal(O.erode(g, img, r), golden[f"sub_{ci}_erode_{ri}"])
        np.testing.assert_array_equal(O.dilate(g, img, r), golden[f"sub_{ci}_dilate_{ri}"])
        np.testing.assert_array_equal(O.erode(g, img, np.float64(r)), golden[f"sub_{ci}_erode64_{ri}"])
        np.testing.assert_array_equal(O.erode(g, img, r, fft=True), golden[f"sub_{ci}_erodefft_{ri}"])
        np.testing.assert_array_equal(O.dilate(g, img, r, fft=True), golden[f"sub_{ci}_dilatefft_{ri}"])
        for mode in ("hybrid", "morph"):
            np.testing.assert_array_equal(O.porosimetry(g, img, r, mode=mode), golden[f"sub_{ci}_por_{mode}_{ri}"])


@pytest.mark.parametrize("ci", range(8))
def test_cc_golden(golden, golden_meta, ci):
    case = golden_meta["cc_cases"][ci]
    g = geom_from_meta(O, case["geom"])
    lbl, n = O.connect_components(golden[f"cc_{ci}_in"], g)
    np.testing.assert_array_equal(lbl, golden[f"cc_{ci}_out"])
    assert n == case["count"]


def test_inlet_outlet_and_drainage_golden(golden, golden_meta):
    g = geom_from_meta(O, golden_meta["drain_geom"])
    img = O.gen_pm_spheres_domain(g, golden["drain_spheres"])
    np.testing.assert_array_equal(img, golden["drain_img"])
    np.testing.assert_array_equal(O.inlet_connected_img(g, img), golden["drain_inlet_img"])
    np.testing.assert_array_equal(O.outlet_connected_img(g, img), golden["drain_outlet_img"])
    np.testing.assert_array_equal(O.inlet_outlet_connected_img(g, img), golden["drain_io_img"])
    np.testing.assert_array_equal(O.isolated_img(g, img), golden["drain_iso_img"])
    sat, mp_img = O.drainage(g, img, list(golden["drain_pcs"]))
    np.testing.assert_array_equal(sat, golden["drain_sat"])
    for meth, key in (("contact_angle", "drain_sat_ca"), ("extended_contact_angle", "drain_sat_eca")):
        sat, mp_img_c = O.drainage(g, img, list(golden["drain_pcs"]), contact_angle=30.0, method=meth)
        np.testing.assert_array_equal(sat, golden[key])
        np.testing.assert_array_equal(mp_img_c, golden[key + "_img"])
    np.testing.assert_array_equal(mp_img, golden["drain_mp_img"])
    np.testing.assert_array_equal(O.porosimetry(g, img, 0.1, inlet=True), golden["drain_por_r"])
    np.testing.assert_array_equal(O.pore_size_distribution(g, img, [0.03, 0.06, 0.09, 0.12]), golden["drain_psd"])
    for mode in ("hybrid", "morph"):
        sat, _ = O.drainage(g, img, list(golden["drain_pcs"]), mode=mode)
        np.testing.assert_array_equal(sat, golden[f"drain_sat_{mode}"])


def test_inkbottle_golden(golden, golden_meta):
    g = geom_from_meta(O, golden_meta["ink_geom"])
    sat, _ = O.drainage(g, golden["ink_img"], list(golden["ink_pcs"]))
    np.testing.assert_array_equal(sat, golden["ink_sat_distance"])
    # the reference test's own expected curve (6 decimals)
    np.testing.assert_array_almost_equal(sat, golden["ink_sat_expected"])
    sat_h, _ = O.drainage(g, golden["ink_img"], list(golden["ink_pcs"]), mode="hybrid")
    np.testing.assert_array_equal(sat_h, golden["ink_sat_hybrid"])
    np.testing.assert_array_almost_equal(sat_h, golden["ink_sat_expected"])


def test_sphere_kat(golden):
    g = O.Geom((10, 10, 10))
    img = O.gen_pm_spheres_domain(g, np.array([[0.5, 0.5, 0.5, 0.25]]))
    np.testing.assert_array_equal(img, golden["sphere10_img"])
    assert int(img.sum()) == 944


# ---------------------------------------------------------------------------
# line-by-line against the reference's own compiled kernels
# ---------------------------------------------------------------------------

def _reflib():
    # built by the build recipe where the reference sources are mounted, or
    # from $PMMOTO_REF_SRC
    so = os.path.join(OB.OUT, "libpmref.so")
    if not os.path.exists(so):
        so = OB.build_reference()
    if so is None or not os.path.exists(so):
        pytest.skip("reference sources not available to build libpmref")
    L = ctypes.CDLL(so)
    P = ctypes.c_void_p
    L.ref_squared_edt_1d.argtypes = [P, P, ctypes.c_int, ctypes.c_long, ctypes.c_float, ctypes.c_float, ctypes.c_float]
    L.ref_parabolic_1d.argtypes = [P, ctypes.c_int, ctypes.c_float, ctypes.c_long, P, ctypes.c_int, P, ctypes.c_int]
    L.ref_boundary_hull.argtypes = [P, ctypes.c_int, ctypes.c_float, ctypes.c_long, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, P]
    L.ref_boundary_hull.restype = ctypes.c_int
    L.ref_unique_pairs.argtypes = [P, ctypes.c_int64, P]
    L.ref_unique_pairs.restype = ctypes.c_int64
    L.ref_spheres.argtypes = [P, ctypes.c_long, P, P, P, P, ctypes.c_long, ctypes.c_long, ctypes.c_long]
    return L


def test_lines_match_reference_kernels():
    L = _reflib()
    ol = O.lib()
    rng = np.random.default_rng(7)
    P = O._ptr
    for trial in range(400):
        n = int(rng.integers(1, 70))
        res = np.float32(rng.choice([1.0, 0.01, 1 / 3, 0.5, 233.0, 0.32325245]))
        img = rng.integers(0, 3 if trial % 3 == 0 else 2, n).astype(np.uint8)
        lc = np.float32(rng.choice([np.inf, rng.integers(1, 9)]))
        uc = np.float32(rng.choice([np.inf, rng.integers(1, 9)]))
        a = np.zeros(n, np.float32)
        b = np.zeros(n, np.float32)
        L.ref_squared_edt_1d(P(img), P(a), n, 1, float(res), float(lc), float(uc))
        ol.or_edt_pass0_line(P(img), P(b), n, 1, float(res), float(lc), float(uc))
        np.testing.assert_array_equal(a, b)
        a[a == np.inf] = np.finfo(np.float32).max
        # envelope with random imported hulls
        nl, nu = int(rng.integers(0, 4)), int(rng.integers(0, 4))
        lo = (O.OrHull * max(nl, 1))()
        up = (O.OrHull * max(nu, 1))()
        for j in range(nl):
            lo[j].vertex = -int(rng.integers(1, 6)) - 3 * j
            lo[j].height = float(rng.integers(0, 30)) * float(res) * float(res)
            lo[j].range = float(-rng.random() * 3 - 3 * j)
        for j in range(nu):
            up[j].vertex = int(rng.integers(0, 3)) + 3 * j
            up[j].height = float(rng.integers(0, 30)) * float(res) * float(res)
            up[j].range = 0.0
        x = a.copy()
        y = a.copy()
        L.ref_parabolic_1d(P(x), n, float(res), 1, ctypes.addressof(lo), nl, ctypes.addressof(up), nu)
        ol.or_parabolic_line(P(y), n, float(res), 1, ctypes.addressof(lo), nl, ctypes.addressof(up), nu)
        np.testing.assert_array_equal(x, y)
        if n >= 2:
            for fwd in (0, 1):
                for corr in (0, -n, 3):
                    hr = (O.OrHull * 8)()
                    ho = (O.OrHull * 8)()
                    x = a.copy()
                    y = a.copy()
                    cr = L.ref_boundary_hull(P(x), n, float(res), 1, 4, corr, fwd, ctypes.addressof(hr))
                    co = ol.or_boundary_hull(P(y), n, float(res), 1, 4, corr, fwd, ctypes.addressof(ho))
                    assert cr == co
                    for j in range(cr):
                        assert (hr[j].vertex, hr[j].height, hr[j].range) == (ho[j].vertex, ho[j].height, ho[j].range)


def test_unique_pairs_and_spheres_match_reference():
    L = _reflib()
    rng = np.random.default_rng(11)
    P = O._ptr
    pairs = rng.integers(0, 50, (3000, 2)).astype(np.uint64)
    out = np.zeros_like(pairs)
    m = L.ref_unique_pairs(P(pairs), pairs.shape[0], P(out))
    np.testing.assert_array_equal(out[:m], O.unique_pairs(pairs))
    sph = np.c_[rng.random((40, 3)), rng.uniform(0.02, 0.2, 40)]
    cx, cy, cz = (np.linspace(0.01, 0.99, k) for k in (11, 13, 17))
    img = np.zeros((11, 13, 17), np.uint8)
    L.ref_spheres(P(sph), 40, P(cx), P(cy), P(cz), P(img), 11, 13, 17)
    np.testing.assert_array_equal(img, O.sphere_fill(sph, (cx, cy, cz)))
