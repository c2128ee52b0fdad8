"""Generate the golden fixtures in this folder from the PMMoTo reference.

Run in a container where the reference is installed under ``baseline/_ref``
(``python -m pip install --no-index --no-build-isolation --no-deps --target
baseline/_ref <pmmoto source>``)::

    python tests/golden/make_golden.py

Every fixture is an output of the reference's own public functions
(``pmmoto.filters.*``, ``pmmoto.domain_generation.*``) on seeded inputs; the
stand-ins it runs under are described in ``refshim.py``.  The known-answer
vectors of the reference's tests are read from its test files (the
``capillary_pressure`` / ``w_saturation_expected`` lists of
tests/applications/test_drainage_inkbottle.py) rather than re-typed.

Writes ``golden_small.npz`` (arrays for small cases, bit-exact compares) and
``golden_meta.json`` (sha256 digests and scalars for the full-size
128^3 periodic sphere-pack case).
"""

from __future__ import annotations

import hashlib
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refshim  # noqa: E402

# the reference's test directory (its fixture scripts are read in place)
REF_TESTS = os.environ.get("PMMOTO_REF_TESTS")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    if not REF_TESTS or not os.path.isdir(REF_TESTS):
        raise SystemExit("set PMMOTO_REF_TESTS to the reference's tests directory")
    pm = refshim.load()
    if pm is None:
        raise SystemExit("reference not importable; install it under baseline/_ref first")
    BT = pm.BoundaryType
    P, E, W = (BT.PERIODIC,) * 2, (BT.END,) * 2, (BT.WALL,) * 2
    dist = pm.filters.distance
    morph = pm.filters.morphological_operators
    ccm = pm.filters.connected_components
    out: dict[str, np.ndarray] = {}
    meta: dict = {"cases": {}}

    def put(name, arr):
        out[name] = np.asarray(arr)

    def geom_meta(vox, bts, box, inlet=((0, 0),) * 3, outlet=((0, 0),) * 3, rv=0):
        return {"voxels": list(vox), "boundary_types": [[b.value for b in bt] for bt in bts],
                "box": [list(map(float, b)) for b in box], "inlet": [list(map(int, i)) for i in inlet],
                "outlet": [list(map(int, o)) for o in outlet], "reservoir_voxels": rv}

    # ---- 1-D known answers (tests/filters/test_edt.py) -------------------
    line = np.array([1, 1, 0, 0, 1, 1, 0, 1, 1, 1, 1, 1, 1, 0, 1], dtype=np.uint8)
    put("kat_pass0_in", line)
    put("kat_pass0_out", dist._distance.determine_initial_envelope_1d(
        img=line, start=0, size=len(line), lower_corrector=np.inf, upper_corrector=np.inf))
    line2 = np.array([1, 1, 0, 1, 1, 1, 1, 1, 1], dtype=np.uint8)
    put("kat_pass0c_in", line2)
    put("kat_pass0c_out_11", dist._distance.determine_initial_envelope_1d(
        img=line2, start=0, size=len(line2), lower_corrector=1, upper_corrector=1))
    put("kat_pass0c_out_24", dist._distance.determine_initial_envelope_1d(
        img=line2, start=0, size=len(line2), lower_corrector=2, upper_corrector=4))
    hull_in = np.array([4, np.inf, 0, np.inf, np.inf, np.inf, 4, 6, 16], dtype=np.float32)
    put("kat_hull_in", hull_in)
    hull_cases = [(0, 9, 2, True), (0, 9, 1, False), (0, 9, 4, False), (0, 8, 5, False)]
    hulls = []
    for (s, e, nh, fwd) in hull_cases:
        h = dist._distance.get_boundary_hull_1d(img=hull_in.copy(), start=s, end=e, resolution=1.0,
                                               num_hull=nh, forward=fwd)
        hulls.append([[int(x["vertex"]), float(x["height"]), float(x["range"])] for x in h])
    meta["kat_hulls"] = {"cases": hull_cases, "hulls": hulls}

    # ---- 3-D edt3d on random images -------------------------------------
    rng = np.random.default_rng(20261203)
    edt_cases = []
    for ci, (shape, p0, per, res) in enumerate([
        ((17, 23, 29), 0.1, (False, False, False), (1.0, 1.0, 1.0)),
        ((17, 23, 29), 0.1, (True, True, True), (1.0, 1.0, 1.0)),
        ((20, 18, 22), 0.05, (True, False, True), (0.01, 0.01, 0.01)),
        ((16, 19, 21), 0.15, (True, True, True), (1.0, 0.32325245, 233.0)),
        ((24, 24, 24), 0.02, (False, True, True), (1.0 / 24, 1.0 / 24, 1.0 / 24)),
        ((9, 40, 33), 0.2, (True, True, False), (0.5, 0.5, 0.5)),
    ]):
        img = (rng.random(shape) >= p0).astype(np.uint8)
        put(f"edt3d_{ci}_in", img)
        put(f"edt3d_{ci}_out", dist.edt3d(img, periodic=per, resolution=res, squared=True))
        edt_cases.append({"periodic": list(per), "resolution": list(res)})
    # multi-label pass-0 resets
    lab = rng.integers(0, 4, (13, 15, 17)).astype(np.uint8)
    put("edt3d_labels_in", lab)
    put("edt3d_labels_out", dist.edt3d(lab, squared=True))
    meta["edt3d_cases"] = edt_cases
    # edt2d
    img2 = (rng.random((37, 41)) >= 0.1).astype(np.uint8)
    put("edt2d_in", img2)
    put("edt2d_out_p", dist.edt2d(img2, periodic=(True, True)))
    put("edt2d_out_n", dist.edt2d(img2))

    # ---- subdomain workflows ----------------------------------------------
    sub_cases = []
    for ci, (vox, bts, nsph, radii) in enumerate([
        ((32, 32, 32), (P, P, P), 60, (0.05, 0.0625, 0.1)),
        ((30, 24, 36), (E, W, W), 60, (0.05, 0.1)),
        ((24, 28, 20), (P, E, W), 40, (0.05, 0.09)),
        ((20, 26, 30), (W, P, P), 40, (0.0625,)),
        ((30, 30, 30), (E, E, E), 50, (1.0 / 15,)),
    ]):
        box = tuple((0.0, v / 32) for v in vox)
        sd = pm.initialize(vox, box=box, boundary_types=bts)
        sph = np.c_[rng.random((nsph, 3)) * np.array([b[1] for b in box]), rng.uniform(0.03, 0.12, nsph)]
        pmo = pm.domain_generation.gen_pm_spheres_domain(sd, sph)
        put(f"sub_{ci}_spheres", sph)
        put(f"sub_{ci}_img", pmo.img)
        put(f"sub_{ci}_edt", dist.edt(pmo.img, sd))
        lbl, n = ccm.connect_components(pmo.img, sd)
        put(f"sub_{ci}_cc", lbl)
        for ri, r in enumerate(radii):
            put(f"sub_{ci}_erode_{ri}", morph.erode(sd, pmo.img, r))
            put(f"sub_{ci}_dilate_{ri}", morph.dilate(sd, pmo.img, r))
            put(f"sub_{ci}_erode64_{ri}", morph.erode(sd, pmo.img, np.float64(r)))
            put(f"sub_{ci}_erodefft_{ri}", morph.erode(sd, pmo.img, r, fft=True))
            put(f"sub_{ci}_dilatefft_{ri}", morph.dilate(sd, pmo.img, r, fft=True))
            for mode in ("hybrid", "morph"):
                put(f"sub_{ci}_por_{mode}_{ri}", pm.filters.porosimetry.porosimetry(sd, pmo, r, mode=mode))
        sub_cases.append({"geom": geom_meta(vox, bts, box), "radii": list(radii), "cc_count": int(n)})
    meta["sub_cases"] = sub_cases

    # ---- connected components with many labels -------------------------------
    cc_cases = []
    for ci, (vox, bts, kind) in enumerate([
        ((12, 14, 10), (P, P, P), "rand"), ((12, 14, 10), (P, E, E), "rand"),
        ((12, 14, 10), (E, E, P), "arange"), ((12, 14, 10), (P, P, E), "multi"),
        ((12, 14, 10), (P, W, P), "rand"), ((12, 14, 10), (E, E, E), "multi"),
        ((10, 10, 10), (P, E, E), "arange"), ((10, 10, 10), (P, P, P), "arange"),
    ]):
        box = tuple((0.0, v / 16) for v in vox)
        sd = pm.initialize(vox, box=box, boundary_types=bts)
        if kind == "rand":
            img = (rng.random(sd.voxels) > 0.72).astype(np.uint8)
        elif kind == "multi":
            img = rng.integers(0, 3, sd.voxels).astype(np.uint8)
        else:
            img = np.arange(np.prod(sd.voxels), dtype=np.int64).reshape(sd.voxels)
        lbl, n = ccm.connect_components(img, sd)
        put(f"cc_{ci}_in", img)
        put(f"cc_{ci}_out", lbl)
        cc_cases.append({"geom": geom_meta(vox, bts, box), "count": int(n)})
    meta["cc_cases"] = cc_cases

    # ---- inlet / outlet selection and drainage on a small pack -----------------
    vox = (40, 40, 40)
    box = ((0.0, 1.0),) * 3
    inlet, outlet = ((1, 0), (0, 0), (0, 0)), ((0, 1), (0, 0), (0, 0))
    sd = pm.initialize(vox, box=box, boundary_types=(E, W, W), inlet=inlet, outlet=outlet)
    sph = np.c_[rng.random((150, 3)), rng.uniform(0.03, 0.08, 150)]
    pmo = pm.domain_generation.gen_pm_spheres_domain(sd, sph)
    put("drain_spheres", sph)
    put("drain_img", pmo.img)
    put("drain_inlet_img", ccm.inlet_connected_img(sd, pmo.img))
    put("drain_outlet_img", ccm.outlet_connected_img(sd, pmo.img))
    put("drain_io_img", ccm.inlet_outlet_connected_img(sd, pmo.img))
    put("drain_iso_img", ccm.isolated_img(sd, pmo.img))
    mp = pm.domain_generation.gen_mp_constant(pmo, 2)
    rvox = np.linspace(1, 8, 8)
    pcs = sorted(list(2.0 / (rvox * sd.domain.resolution[0])))
    put("drain_pcs", np.array(pcs))
    put("drain_sat", pm.filters.equilibrium_distribution.drainage(mp, pcs, mode="distance"))
    put("drain_mp_img", mp.img)
    put("drain_por_r", pm.filters.porosimetry.porosimetry(sd, pmo, 0.1, inlet=True, mode="distance"))
    put("drain_psd", pm.filters.porosimetry.pore_size_distribution(
        sd, pmo, radii=[0.03, 0.06, 0.09, 0.12], inlet=False, mode="distance"))
    put("drain_psd_auto", pm.filters.porosimetry.pore_size_distribution(sd, pmo, num_radii=6, mode="distance"))
    mp_h = pm.domain_generation.gen_mp_constant(pmo, 2)
    put("drain_sat_hybrid", pm.filters.equilibrium_distribution.drainage(mp_h, pcs, mode="hybrid"))
    mp_m = pm.domain_generation.gen_mp_constant(pmo, 2)
    put("drain_sat_morph", pm.filters.equilibrium_distribution.drainage(mp_m, pcs, mode="morph"))
    # contact-angle methods (equilibrium_distribution.py:182-289), 30 degrees
    for meth, key in (("contact_angle", "drain_sat_ca"), ("extended_contact_angle", "drain_sat_eca")):
        mp_c = pm.domain_generation.gen_mp_constant(pmo, 2)
        put(key, pm.filters.equilibrium_distribution.drainage(mp_c, pcs, contact_angle=30.0, method=meth,
                                                              mode="distance"))
        put(key + "_img", mp_c.img)
    meta["drain_geom"] = geom_meta(vox, (E, W, W), box, inlet, outlet)

    # ---- ink bottle (tests/applications/test_drainage_inkbottle.py) -------------
    spec = importlib.util.spec_from_file_location(
        "ref_inkbottle", os.path.join(REF_TESTS, "applications", "test_drainage_inkbottle.py"))
    tmod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(tmod)
    mp_ink = tmod.initialize_ink_bottle()
    put("ink_img", mp_ink.porous_media.img)
    put("ink_pcs", np.array(tmod.capillary_pressure, dtype=np.float64))
    put("ink_sat_expected", np.array(tmod.w_saturation_expected, dtype=np.float64))
    put("ink_sat_distance", pm.filters.equilibrium_distribution.drainage(mp_ink, list(tmod.capillary_pressure),
                                                                        mode="distance"))
    mp_ink2 = tmod.initialize_ink_bottle()
    put("ink_sat_hybrid", pm.filters.equilibrium_distribution.drainage(mp_ink2, list(tmod.capillary_pressure)))
    meta["ink_geom"] = geom_meta((140, 30, 30), (E, E, E), ((0.0, 14.0), (-1.5, 1.5), (-1.5, 1.5)),
                                 ((0, 1), (0, 0), (0, 0)), ((1, 0), (0, 0), (0, 0)), 10)

    # ---- sphere voxelisation known answer (test_domain_generation.py) ----------
    sd = pm.initialize((10, 10, 10))
    pm10 = pm.domain_generation.gen_pm_spheres_domain(sd, np.array([[0.5, 0.5, 0.5, 0.25]]))
    put("sphere10_img", pm10.img)

    # ---- full size: 128^3 periodic pack, 400 spheres (r in [0.03, 0.08]) --------
    full = {}
    for seed in (0, 1):
        r2 = np.random.default_rng(seed)
        sph = np.c_[r2.random((400, 3)), r2.uniform(0.03, 0.08, 400)]
        sd = pm.initialize((128,) * 3, boundary_types=(P, P, P))
        pmo = pm.domain_generation.gen_pm_spheres_domain(sd, sph)
        own = np.ascontiguousarray(pmo.img[1:-1, 1:-1, 1:-1])
        e3 = dist.edt3d(own, periodic=(True, True, True))
        es = dist.edt(pmo.img, sd)
        full[str(seed)] = {"img_sha": sha(pmo.img), "edt3d_sha": sha(e3), "edt_sd_sha": sha(es),
                           "porosity": float(np.count_nonzero(own) / own.size),
                           "edt3d_max": float(e3.max())}
    meta["c1_full"] = full

    # ---- periodic sphere images, ownership, trimming, gen_pm_shape --------------
    from pmmoto.domain_generation import _domain_generation as dgen

    r3 = np.random.default_rng(77)
    vox, box = (24, 20, 28), ((0.0, 1.2), (0.0, 1.0), (0.0, 1.4))
    cases = []
    for ci, bts in enumerate([(P, P, P), (P, E, W)]):
        sd = pm.initialize(vox, box=box, boundary_types=bts)
        sph = np.c_[r3.random((40, 3)) * np.array([b[1] for b in box]), r3.uniform(0.05, 0.2, 40)]
        put(f"psph_{ci}_in", sph)
        for key, kw in (("per", dict(add_periodic=True)), ("plain", {}),
                        ("trim", dict(add_periodic=True, trim_intersecting=True)),
                        ("within", dict(trim_within=True))):
            lst = pm.particles.initialize_spheres(sd, sph, **kw)
            put(f"psph_{ci}_{key}", np.asarray(lst.return_np_array(return_own=True)))
            put(f"psph_{ci}_{key}_count", np.array([lst.size(), lst.get_own_count()]))
            if key == "per":
                put(f"psph_{ci}_img", dgen.gen_pm_shape(sd, lst))
        cases.append(geom_meta(vox, bts, box))
    meta["psph_cases"] = cases

    # ---- sphere-pack file reader on a synthetic pack ----------------------------
    import tempfile

    text = "0.0 1.5\n-0.5 0.5\n0.0 2.0\n" + "".join(
        f"{x:.6f} {y:.6f} {z:.6f} {r:.6f}\n" for x, y, z, r in
        np.c_[r3.random((7, 3)) * np.array([1.5, 1.0, 2.0]) - np.array([0.0, 0.5, 0.0]), r3.uniform(0.1, 0.3, 7)])
    with tempfile.NamedTemporaryFile("w", suffix=".out", delete=False) as f:
        f.write(text)
        fname = f.name
    sph_r, dom_r = pm.io.data_read.read_sphere_pack_xyzr_domain(fname)
    os.unlink(fname)
    put("pack_read_spheres", sph_r)
    put("pack_read_domain", np.asarray(dom_r))
    meta["pack_text"] = text

    write_vti(pm)
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)
    with open(os.path.join(HERE, "golden_meta.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", len(out), "arrays")


def write_vti(pm):
    """Image-writer fixtures: the reference's save_img output for the seeded
    cases of vti_cases.py, one .vti file per case under vti/."""
    import vti_cases

    BT = pm.BoundaryType
    for name, kw, imgs in vti_cases.cases():
        kw = dict(kw)
        if kw.pop("boundary_types", None) == "periodic":
            kw["boundary_types"] = ((BT.PERIODIC,) * 2,) * 3
        sd = pm.initialize(**kw)
        extra = {k: v for k, v in imgs.items() if k != "img"}
        pm.io.output.save_img(os.path.join(HERE, "vti", name), sd, imgs["img"],
                              additional_img=extra or None)


if __name__ == "__main__" and "--vti-only" in sys.argv:
    write_vti(refshim.load())
elif __name__ == "__main__":
    main()
