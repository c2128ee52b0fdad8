"""Sphere voxelisation, porosimetry, pore-size distribution and drainage on
the GPU vs the reference fixtures and the oracle."""

import hashlib

import numpy as np
import pytest

from oracle import oracle as O
from tests._helpers import sd_from_meta

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import pmmoto_gb300
    return pmmoto_gb300


def test_sphere_kat(P, golden):
    sd = P.initialize((10, 10, 10))
    pm = P.domain_generation.gen_pm_spheres_domain(sd, np.array([[0.5, 0.5, 0.5, 0.25]]))
    np.testing.assert_array_equal(pm.img, golden["sphere10_img"])
    assert int(pm.img.sum()) == 944


@pytest.mark.parametrize("ci", range(5))
def test_spheres_and_porosimetry_golden(P, golden, golden_meta, ci):
    case = golden_meta["sub_cases"][ci]
    sd = sd_from_meta(case["geom"])
    pm = P.domain_generation.gen_pm_spheres_domain(sd, golden[f"sub_{ci}_spheres"])
    np.testing.assert_array_equal(pm.img, golden[f"sub_{ci}_img"])
    for ri, r in enumerate(case["radii"]):
        for mode in ("hybrid", "morph"):
            np.testing.assert_array_equal(P.filters.porosimetry.porosimetry(sd, pm, r, mode=mode),
                                          golden[f"sub_{ci}_por_{mode}_{ri}"])


def test_c1_sphere_hashes(P, golden_meta):
    for seed, want in golden_meta["c1_full"].items():
        r2 = np.random.default_rng(int(seed))
        sph = np.c_[r2.random((400, 3)), r2.uniform(0.03, 0.08, 400)]
        sd = P.initialize((128,) * 3, boundary_types=(("periodic",) * 2,) * 3)
        pm = P.domain_generation.gen_pm_spheres_domain(sd, sph)
        assert hashlib.sha256(pm.img.tobytes()).hexdigest() == want["img_sha"]


def test_drainage_golden(P, golden, golden_meta):
    sd = sd_from_meta(golden_meta["drain_geom"])
    pm = P.domain_generation.gen_pm_spheres_domain(sd, golden["drain_spheres"])
    np.testing.assert_array_equal(pm.img, golden["drain_img"])
    np.testing.assert_array_equal(P.filters.porosimetry.porosimetry(sd, pm, 0.1, inlet=True, mode="distance"),
                                  golden["drain_por_r"])
    np.testing.assert_array_equal(
        P.filters.porosimetry.pore_size_distribution(sd, pm, radii=[0.03, 0.06, 0.09, 0.12], mode="distance"),
        golden["drain_psd"])
    np.testing.assert_array_equal(P.filters.porosimetry.pore_size_distribution(sd, pm, num_radii=6, mode="distance"),
                                  golden["drain_psd_auto"])
    pcs = list(golden["drain_pcs"])
    mp = P.domain_generation.gen_mp_constant(pm, 2)
    sat = P.filters.equilibrium_distribution.drainage(mp, pcs, mode="distance")
    np.testing.assert_array_equal(sat, golden["drain_sat"])
    np.testing.assert_array_equal(mp.img, golden["drain_mp_img"])
    for mode in ("hybrid", "morph"):
        mp = P.domain_generation.gen_mp_constant(pm, 2)
        np.testing.assert_array_equal(P.filters.equilibrium_distribution.drainage(mp, pcs, mode=mode),
                                      golden[f"drain_sat_{mode}"])
    # contact-angle methods at 30 degrees (the extended one dilates by r cos(theta))
    for meth, key in (("contact_angle", "drain_sat_ca"), ("extended_contact_angle", "drain_sat_eca")):
        mp = P.domain_generation.gen_mp_constant(pm, 2)
        sat = P.filters.equilibrium_distribution.drainage(mp, pcs, contact_angle=30.0, method=meth, mode="distance")
        np.testing.assert_array_equal(sat, golden[key])
        np.testing.assert_array_equal(mp.img, golden[key + "_img"])


def test_inkbottle(P, golden, golden_meta):
    m = golden_meta["ink_geom"]
    sd = sd_from_meta(m)
    pm = P.domain_generation.PorousMedia(sd, golden["ink_img"])
    pcs = list(golden["ink_pcs"])
    for mode, key in (("distance", "ink_sat_distance"), ("hybrid", "ink_sat_hybrid")):
        mp = P.domain_generation.gen_mp_constant(pm, 2)
        sat = P.filters.equilibrium_distribution.drainage(mp, pcs, mode=mode)
        np.testing.assert_array_equal(sat, golden[key])
        np.testing.assert_array_almost_equal(sat, golden["ink_sat_expected"])


@pytest.mark.parametrize("seed", range(3))
def test_drainage_random_vs_oracle(P, seed):
    rng = np.random.default_rng(50 + seed)
    vox = (36, 30, 28)
    box = tuple((0.0, v / 32) for v in vox)
    bts = (("end", "end"), ("wall", "wall"), ("periodic", "periodic")) if seed == 1 else \
        (("end", "end"), ("wall", "wall"), ("wall", "wall"))
    inlet, outlet = ((True, False), (False, False), (False, False)), ((False, True), (False, False), (False, False))
    rv = 3 if seed == 2 else 0
    sd = P.initialize(vox, box=box, boundary_types=bts, inlet=inlet, outlet=outlet, reservoir_voxels=rv)
    g = O.Geom(vox, boundary_types=bts, box=box, inlet=inlet, outlet=outlet, reservoir_voxels=rv)
    sph = np.c_[rng.random((120, 3)) * np.array([b[1] for b in box]), rng.uniform(0.03, 0.09, 120)]
    pm = P.domain_generation.gen_pm_spheres_domain(sd, sph)
    np.testing.assert_array_equal(pm.img, O.gen_pm_spheres_domain(g, sph))
    pcs = sorted(list(2.0 / (np.linspace(1, 7, 9) / 32)))
    mp = P.domain_generation.gen_mp_constant(pm, 2)
    sat = P.filters.equilibrium_distribution.drainage(mp, pcs, mode="distance")
    want, want_img = O.drainage(g, pm.img, pcs)
    np.testing.assert_array_equal(sat, want)
    np.testing.assert_array_equal(mp.img, want_img)


@pytest.mark.parametrize("case", ["many_radii", "unsorted_array", "periodic"])
def test_drainage_growing_selections_vs_oracle(P, case):
    """Many radii: the eroded space and the non-wetting phase keep their
    block union-find from radius to radius; an unsorted pressure array (the
    reference sorts lists only) makes the erosion thresholds rise and fall."""
    rng = np.random.default_rng({"many_radii": 71, "unsorted_array": 72, "periodic": 73}[case])
    vox = (64, 48, 40)
    box = tuple((0.0, v / 32) for v in vox)
    bts = (("end", "end"), ("wall", "wall"), ("wall", "wall"))
    if case == "periodic":
        bts = (("end", "end"), ("periodic", "periodic"), ("periodic", "periodic"))
    inlet, outlet = ((True, False), (False, False), (False, False)), ((False, True), (False, False), (False, False))
    sd = P.initialize(vox, box=box, boundary_types=bts, inlet=inlet, outlet=outlet)
    g = O.Geom(vox, boundary_types=bts, box=box, inlet=inlet, outlet=outlet)
    sph = np.c_[rng.random((260, 3)) * np.array([b[1] for b in box]), rng.uniform(0.03, 0.12, 260)]
    pm = P.domain_generation.gen_pm_spheres_domain(sd, sph)
    pcs = sorted(list(2.0 / (np.linspace(1, 9, 17) / 32)))
    if case == "unsorted_array":
        pcs = np.array(pcs)[rng.permutation(len(pcs))]
    mp = P.domain_generation.gen_mp_constant(pm, 2)
    sat = P.filters.equilibrium_distribution.drainage(mp, pcs, mode="distance")
    want, want_img = O.drainage(g, pm.img, pcs)
    np.testing.assert_array_equal(sat, want)
    np.testing.assert_array_equal(mp.img, want_img)


@pytest.mark.parametrize("ci", range(2))
def test_gen_pm_shape_periodic_images_golden(P, golden, golden_meta, ci):
    """Voxelisation of a sphere list with periodic images (gen_pm_shape)."""
    sd = sd_from_meta(golden_meta["psph_cases"][ci])
    lst = P.particles.initialize_spheres(sd, golden[f"psph_{ci}_in"], add_periodic=True)
    np.testing.assert_array_equal(P.domain_generation.gen_pm_shape(sd, lst), golden[f"psph_{ci}_img"])

