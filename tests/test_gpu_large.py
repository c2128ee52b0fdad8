"""Full-size parity of the benchmarked configurations against digests the
reference itself produced (``tests/golden/make_golden_large.py``).

* 512 x 514 x 514 sphere-pack drainage (the bench workload): the pore image,
  porosity, max distance, the 40 float64 saturations of
  drainage(mode="distance") and the final multiphase image are those the
  reference computed, bit for bit.
* 1024^3 Gaussian-random-field medium (periodic): the medium generated on the
  device has the reference-side digest (the generator is reproducible bit for
  bit), its periodic squared edt3d and its connected components (labels on
  the padded periodic subdomain image, count) equal the reference's.
* drainage(save=True): the .vti files written per capillary pressure are
  byte-identical to the reference's.
"""

import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

pytestmark = pytest.mark.gpu


def _large():
    p = os.path.join(GOLDEN, "golden_large.json")
    if not os.path.exists(p):
        pytest.skip("golden_large.json not generated")
    with open(p) as f:
        return json.load(f)


def _sha_t(t) -> str:
    return hashlib.sha256(np.ascontiguousarray(t.cpu().numpy()).tobytes()).hexdigest()


def test_drainage512_matches_reference():
    import torch

    import bench
    import pmmoto_gb300 as P
    from pmmoto_gb300.filters import equilibrium_distribution as ED

    ref = _large().get("drainage512")
    if ref is None:
        pytest.skip("drainage512 digests not generated")
    sd = P.initialize((bench.N_VOX,) * 3, **bench.geom_kwargs())
    pm = P.domain_generation.gen_pm_spheres_domain(sd, torch.as_tensor(bench.make_pack(1234), device="cuda"))
    assert list(pm.img.shape) == ref["shape"]
    assert _sha_t(pm.img) == ref["img_sha"]
    assert float(pm.porosity) == ref["porosity"]
    assert float(pm.max_distance) == ref["max_distance"]
    pcs, _ = bench.radii_for(sd.domain.resolution[0])
    assert [float(p) for p in pcs] == ref["pcs"]
    mp = P.domain_generation.gen_mp_constant(pm, 2)
    sat = ED.drainage(mp, pcs, mode="distance")
    assert [float(s) for s in sat] == ref["saturation"]
    assert _sha_t(mp.img) == ref["mp_sha"]


def test_grf1024_edt_and_labels_match_reference():
    import torch

    import pmmoto_gb300 as P
    from pmmoto_gb300.domain_generation import grf
    from pmmoto_gb300.filters import connected_components as CC
    from pmmoto_gb300.filters import distance as D

    ref = _large().get("grf1024")
    if ref is None or "labels_sha" not in ref:
        pytest.skip("grf1024 digests not generated")
    n = ref["n"]
    own = grf.gen_grf_medium(n)
    assert _sha_t(own) == ref["own_sha"]
    e2 = D.edt3d(own, periodic=(True, True, True), squared=True)
    assert _sha_t(e2) == ref["edt3d_sq_sha"]
    del e2
    idx = (torch.arange(-1, n + 1, device="cuda") % n)
    img = own[idx][:, idx][:, :, idx].contiguous()  # periodic halo of one voxel
    del own
    assert _sha_t(img) == ref["padded_sha"]
    sd = P.initialize((n,) * 3, boundary_types=(("periodic", "periodic"),) * 3)
    lbl, count = CC.connect_components(img, sd)
    assert int(count) == ref["label_count"]
    assert _sha_t(lbl) == ref["labels_sha"]


def test_drainage_save_writes_reference_files(tmp_path):
    import torch

    import pmmoto_gb300 as P
    from pmmoto_gb300.filters import equilibrium_distribution as ED

    ref = _large().get("drain_save")
    if ref is None:
        pytest.skip("drain_save digests not generated")
    sd = P.initialize(tuple(ref["voxels"]), box=tuple(tuple(b) for b in ref["box"]),
                      boundary_types=(("end", "end"), ("wall", "wall"), ("wall", "wall")),
                      inlet=((True, False), (False, False), (False, False)),
                      outlet=((False, True), (False, False), (False, False)))
    pm = P.domain_generation.gen_pm_spheres_domain(sd, torch.as_tensor(np.array(ref["spheres"]), device="cuda"))
    mp = P.domain_generation.gen_mp_constant(pm, 2)
    folder = str(tmp_path / "out")
    sat = ED.drainage(mp, ref["pcs"], mode="distance", save=True, out_folder=folder)
    assert [float(s) for s in sat] == ref["saturation"]
    got = {}
    for name in sorted(os.listdir(folder)):
        with open(os.path.join(folder, name), "rb") as f:
            got[name] = hashlib.sha256(f.read()).hexdigest()
    assert got == ref["files"]
    mp2 = P.domain_generation.gen_mp_constant(pm, 2)
    assert [float(s) for s in ED.drainage(mp2, ref["pcs"], mode="distance")] == ref["saturation"]
