"""Generate the full-size golden digests (``golden_large.json``) from the
PMMoTo reference itself, for the benchmarked configurations.

Run where the reference is installed under ``baseline/_ref`` (see
``make_golden.py``); each case is slow on the CPU (minutes) and is run on
its own::

    python tests/golden/make_golden_large.py drainage512   # 512x514x514 pack, 40 radii
    python tests/golden/make_golden_large.py grf1024       # 1024^3 periodic EDT + labels
    python tests/golden/make_golden_large.py save          # drainage(save=True) files

Cases (every output comes from the reference's public functions, under the
stand-ins of ``refshim.py``; CC label numbering therefore rests on the cc3d
stand-in, partitions and counts do not):

* ``drainage512`` -- the plain-drainage configuration exactly as ``bench.py``
  builds it: ``bench.make_pack(1234)`` (3,000 spheres, radii U[0.02, 0.05])
  voxelised on ``initialize((512,)*3)`` with walls on y/z, inlet x-, outlet
  x+ (padded 512 x 514 x 514), then ``drainage(gen_mp_constant(pm, 2), pcs,
  mode="distance")`` over the 40 capillary pressures of
  ``bench.radii_for``.  Stored: digests of the pore image and of the final
  multiphase image, porosity, max distance, the 40 float64 saturations and
  the reference's CPU time.
* ``grf1024`` -- the large EDT + CC configuration: the 1024^3 Gaussian random
  field medium of ``grf.py`` (porosity 0.35, periodic), its periodic
  ``edt3d(squared=True)`` and, on the periodic subdomain's padded image,
  ``connect_components``.  Stored: digests of the medium, the squared EDT and
  the labels, the label count and CPU times.
* ``save`` -- ``drainage(..., save=True)`` on a small pack: the digests of the
  ``.vti`` files the reference writes per capillary pressure.
"""

from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)
import refshim  # noqa: E402

OUT = os.path.join(HERE, "golden_large.json")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _load_out() -> dict:
    if os.path.exists(OUT):
        with open(OUT) as f:
            return json.load(f)
    return {}


def _store(key: str, val) -> None:
    d = _load_out()
    d[key] = val
    with open(OUT, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
        f.write("\n")


def case_drainage512(pm):
    import bench

    BT = pm.BoundaryType
    E, W = (BT.END,) * 2, (BT.WALL,) * 2
    sd = pm.initialize((bench.N_VOX,) * 3, box=((0.0, 1.0),) * 3, boundary_types=(E, W, W),
                       inlet=((True, False), (False, False), (False, False)),
                       outlet=((False, True), (False, False), (False, False)))
    sph = bench.make_pack(1234)
    t0 = time.perf_counter()
    pmo = pm.domain_generation.gen_pm_spheres_domain(sd, sph)
    t_vox = time.perf_counter() - t0
    pcs, _ = bench.radii_for(sd.domain.resolution[0])
    mp = pm.domain_generation.gen_mp_constant(pmo, 2)
    t0 = time.perf_counter()
    dmax = float(pmo.max_distance)
    t_dmax = time.perf_counter() - t0
    t0 = time.perf_counter()
    sat = pm.filters.equilibrium_distribution.drainage(mp, pcs, mode="distance")
    t_drain = time.perf_counter() - t0
    rec = {"shape": list(pmo.img.shape), "img_sha": sha(pmo.img), "porosity": float(pmo.porosity),
           "max_distance": dmax, "pcs": [float(p) for p in pcs], "saturation": [float(s) for s in sat],
           "mp_sha": sha(mp.img), "cpu_s": {"voxelise": t_vox, "max_distance": t_dmax, "drainage": t_drain},
           "cpu": "reference on 1 x86 core of the fixture container"}
    _store("drainage512", rec)
    print(json.dumps({k: v for k, v in rec.items() if k not in ("pcs", "saturation")}))


def case_grf1024(pm):
    import grf

    BT = pm.BoundaryType
    P = (BT.PERIODIC,) * 2
    n = grf.N_GRF
    t0 = time.perf_counter()
    own = grf.grf_medium_host(n)
    t_gen = time.perf_counter() - t0
    rec = {"n": n, "own_sha": sha(own), "porosity": float(np.count_nonzero(own) / own.size),
           "generator": grf.DESCRIPTION}
    _store("grf1024", rec)
    dist = pm.filters.distance
    t0 = time.perf_counter()
    e2 = dist.edt3d(own, periodic=(True, True, True), squared=True)
    rec["cpu_s"] = {"generate": t_gen, "edt3d": time.perf_counter() - t0}
    rec["edt3d_sq_sha"] = sha(e2)
    rec["edt3d_sq_max"] = float(e2.max())
    del e2
    _store("grf1024", rec)
    sd = pm.initialize((n,) * 3, box=((0.0, 1.0),) * 3, boundary_types=(P, P, P))
    img = np.pad(own, 1, mode="wrap")  # periodic halo: copies of the opposite own layers
    del own
    rec["padded_sha"] = sha(img)
    t0 = time.perf_counter()
    lbl, count = pm.filters.connected_components.connect_components(img, sd)
    rec["cpu_s"]["connect_components"] = time.perf_counter() - t0
    rec["labels_sha"] = sha(lbl)
    rec["label_count"] = int(count)
    rec["cpu"] = "reference on 1 x86 core of the fixture container (cc3d stand-in: scipy.ndimage.label)"
    _store("grf1024", rec)
    print(json.dumps(rec))


def case_save(pm):
    BT = pm.BoundaryType
    E, W = (BT.END,) * 2, (BT.WALL,) * 2
    vox = (24, 20, 22)
    box = tuple((0.0, v / 32) for v in vox)
    sd = pm.initialize(vox, box=box, boundary_types=(E, W, W),
                       inlet=((True, False), (False, False), (False, False)),
                       outlet=((False, True), (False, False), (False, False)))
    rng = np.random.default_rng(5)
    sph = np.c_[rng.random((40, 3)) * np.array([b[1] for b in box]), rng.uniform(0.04, 0.09, 40)]
    pmo = pm.domain_generation.gen_pm_spheres_domain(sd, sph)
    mp = pm.domain_generation.gen_mp_constant(pmo, 2)
    rvox = np.array([1.0, 1.5, 2.5, 4.0])
    pcs = sorted(list(2.0 / (rvox * sd.domain.resolution[0])))
    with tempfile.TemporaryDirectory() as td:
        folder = os.path.join(td, "out")
        sat = pm.filters.equilibrium_distribution.drainage(mp, pcs, mode="distance", save=True, out_folder=folder)
        files = {}
        for name in sorted(os.listdir(folder)):
            with open(os.path.join(folder, name), "rb") as f:
                files[name] = hashlib.sha256(f.read()).hexdigest()
    rec = {"voxels": list(vox), "box": [list(b) for b in box], "spheres": sph.tolist(), "pcs": [float(p) for p in pcs],
           "saturation": [float(s) for s in sat], "files": files}
    _store("drain_save", rec)
    print(json.dumps(rec)[:400])


def main():
    pm = refshim.load()
    if pm is None:
        raise SystemExit("reference not importable; install it under baseline/_ref first")
    cases = {"drainage512": case_drainage512, "grf1024": case_grf1024, "save": case_save}
    for name in sys.argv[1:] or list(cases):
        cases[name](pm)


if __name__ == "__main__":
    main()
