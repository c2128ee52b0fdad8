"""Sphere lists (periodic images, ownership, trimming) and the sphere-pack
reader against fixtures made by the reference itself."""

import numpy as np
import pytest

from tests._helpers import sd_from_meta


@pytest.mark.parametrize("ci", range(2))
def test_sphere_lists_golden(golden, golden_meta, ci):
    from pmmoto_gb300 import particles

    sd = sd_from_meta(golden_meta["psph_cases"][ci])
    sph = golden[f"psph_{ci}_in"]
    for key, kw in (("per", dict(add_periodic=True)), ("plain", {}),
                    ("trim", dict(add_periodic=True, trim_intersecting=True)), ("within", dict(trim_within=True))):
        lst = particles.initialize_spheres(sd, sph, **kw)
        np.testing.assert_array_equal(lst.return_np_array(return_own=True), golden[f"psph_{ci}_{key}"])
        assert [lst.size(), lst.get_own_count()] == list(golden[f"psph_{ci}_{key}_count"])


def test_sphere_list_errors():
    from pmmoto_gb300 import particles

    with pytest.raises(ValueError):
        particles.SphereList(np.zeros((0, 3)), np.zeros(0))


def test_sphere_pack_reader_golden(golden, golden_meta, tmp_path):
    from pmmoto_gb300.io import read_sphere_pack_xyzr_domain

    f = tmp_path / "pack.out"
    f.write_text(golden_meta["pack_text"])
    sph, dom = read_sphere_pack_xyzr_domain(str(f))
    np.testing.assert_array_equal(sph, golden["pack_read_spheres"])
    np.testing.assert_array_equal(np.asarray(dom), golden["pack_read_domain"])
    bad = tmp_path / "bad.out"
    bad.write_text(golden_meta["pack_text"] + "1.0 2.0 3.0\n")
    with pytest.raises(ValueError):
        read_sphere_pack_xyzr_domain(str(bad))
    with pytest.raises(SystemExit):
        read_sphere_pack_xyzr_domain(str(tmp_path / "missing.out"))
