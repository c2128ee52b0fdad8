"""Image writer: byte-identical to the reference's save_img output
(fixtures written by tests/golden/make_golden.py from the reference itself)."""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import vti_cases  # noqa: E402


@pytest.mark.parametrize("case", vti_cases.cases(), ids=lambda c: c[0])
def test_save_img_matches_reference_bytes(tmp_path, case):
    import pmmoto_gb300 as P

    name, kw, imgs = case
    kw = dict(kw)
    if kw.pop("boundary_types", None) == "periodic":
        kw["boundary_types"] = ((P.BoundaryType.PERIODIC,) * 2,) * 3
    sd = P.initialize(**kw)
    extra = {k: v for k, v in imgs.items() if k != "img"}
    P.io.output.save_img(str(tmp_path / "sub" / name), sd, imgs["img"], additional_img=extra or None)
    got = (tmp_path / "sub" / f"{name}.vti").read_bytes()
    want = open(os.path.join(HERE, "golden", "vti", f"{name}.vti"), "rb").read()
    assert got == want


def test_save_img_errors(tmp_path):
    import pmmoto_gb300 as P

    sd = P.initialize((10, 10, 10))
    img = np.zeros(sd.voxels)
    P.io.output.save_img(str(tmp_path / "test_img"), sd, img)
    assert (tmp_path / "test_img.vti").exists()
    with pytest.raises(ValueError):
        P.io.output.save_img(str(tmp_path / "test_img"), sd, img, additional_img={"err_img": np.zeros((5, 5, 5))})
    with pytest.raises(TypeError):
        P.io.output.save_img(str(tmp_path / "test_img"), sd, img, additional_img={"img2": 4.0})
