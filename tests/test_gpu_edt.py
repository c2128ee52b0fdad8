"""EDT parity: CUDA path vs the oracle and the reference's golden fixtures."""

import hashlib
import json

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def D():
    from pmmoto_gb300.filters import distance
    return distance


def test_kat_lines(D):
    # the 1-D known answers are single lines of a (1, 1, n) volume along axis 2
    img = np.array([1, 1, 0, 0, 1, 1, 0, 1, 1, 1, 1, 1, 1, 0, 1], dtype=np.uint8)
    out = D.edt3d(img.reshape(len(img), 1, 1), squared=True).ravel()
    np.testing.assert_array_equal(out, O.initial_envelope_1d(img))


@pytest.mark.parametrize("ci", range(6))
def test_edt3d_golden(D, golden, golden_meta, ci):
    c = golden_meta["edt3d_cases"][ci]
    out = D.edt3d(golden[f"edt3d_{ci}_in"], periodic=c["periodic"], resolution=c["resolution"], squared=True)
    np.testing.assert_array_equal(out, golden[f"edt3d_{ci}_out"])


def test_edt3d_labels(D, golden):
    np.testing.assert_array_equal(D.edt3d(golden["edt3d_labels_in"], squared=True), golden["edt3d_labels_out"])


def test_edt2d(D, golden):
    np.testing.assert_array_equal(D.edt2d(golden["edt2d_in"], periodic=(True, True)), golden["edt2d_out_p"])
    np.testing.assert_array_equal(D.edt2d(golden["edt2d_in"]), golden["edt2d_out_n"])


@pytest.mark.parametrize("seed", range(12))
def test_edt3d_random_vs_oracle(D, seed):
    rng = np.random.default_rng(100 + seed)
    shape = tuple(int(x) for x in rng.integers(1, 45, 3))
    p0 = float(rng.choice([0.0, 0.01, 0.1, 0.4, 0.9, 1.0]))
    img = (rng.random(shape) >= p0).astype(np.uint8)
    if seed % 4 == 3:
        img = rng.integers(0, 4, shape).astype(np.uint8)
    per = tuple(bool(x) for x in rng.integers(0, 2, 3))
    res = [(1.0, 1.0, 1.0), (0.01, 0.01, 0.01), (1.0, 0.32325245, 233.0), (1 / 3, 1 / 3, 1 / 7)][seed % 4]
    got = D.edt3d(img, periodic=per, resolution=res, squared=True)
    want = O.edt3d(img, periodic=per, resolution=res, squared=True)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(D.edt3d(img, periodic=per, resolution=res), np.sqrt(want))


@pytest.mark.parametrize("seed", range(16))
def test_edt3d_periodic_pow2_vs_oracle(D, seed):
    """Periodic axes with power-of-two voxels: windowed exact minima in the
    line interiors, the float envelope on the end segments and on lines
    without a solid voxel."""
    rng = np.random.default_rng(300 + seed)
    shape = tuple(int(x) for x in rng.integers(1, 61, 3))
    p0 = float([0.02, 0.1, 0.3, 0.5, 0.7, 0.9, 0.98, 0.999][seed % 8])
    img = (rng.random(shape) >= p0).astype(np.uint8)
    if seed % 5 == 4:
        img = np.where(img > 0, rng.integers(1, 4, shape), 0).astype(np.uint8)
    per = tuple(bool(x) for x in rng.integers(0, 2, 3))
    if not any(per):
        per = (True, True, True)
    res = [(1.0, 1.0, 1.0), (0.5, 0.5, 0.5), (1 / 128, 1 / 128, 1 / 128), (0.25, 1.0, 2.0)][seed % 4]
    got = D.edt3d(img, periodic=per, resolution=res, squared=True)
    want = O.edt3d(img, periodic=per, resolution=res, squared=True)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("seed", range(10))
def test_edt3d_line_pairs_vs_oracle(D, seed):
    """Envelope passes over pairs of lines (even extents): packed direct
    minima within +-12, the per-voxel scan beyond it, for clamped heights
    (lines without a solid voxel) and near periodic line ends; lines longer
    than one 256-voxel segment or one 128-column tile; porosities from 30 %
    to 99.9 %."""
    rng = np.random.default_rng(900 + seed)
    shape = [(300, 90, 64), (70, 520, 32), (64, 64, 128), (33, 270, 18), (260, 40, 2)][seed % 5]
    p0 = float([0.7, 0.3, 0.05, 0.01, 0.001][seed % 5 if seed < 5 else (seed + 2) % 5])
    img = (rng.random(shape) >= p0).astype(np.uint8)
    per = [(True, True, True), (False, False, False), (True, False, True), (False, True, False)][seed % 4]
    res = [(1.0, 1.0, 1.0), (0.5, 0.5, 0.5), (1 / 128, 1 / 128, 1 / 128)][seed % 3]
    for squared in (True, False):
        got = D.edt3d(img, periodic=per, resolution=res, squared=squared)
        want = O.edt3d(img, periodic=per, resolution=res, squared=squared)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("seed", range(12))
def test_edt3d_pass0_quads_vs_oracle(D, seed):
    """Pass 0 on four lines per thread (the last extent a multiple of 4):
    zeros, restarts between adjacent voxels of different values, periodic
    correctors, long runs without a zero; power-of-two and other voxel
    sizes."""
    rng = np.random.default_rng(1200 + seed)
    shape = [(64, 48, 40), (33, 20, 128), (130, 7, 12), (5, 64, 4)][seed % 4]
    p0 = float([0.5, 0.1, 0.01, 0.9, 0.3, 0.0][seed % 6])
    img = (rng.random(shape) >= p0).astype(np.uint8)
    if seed % 3 == 1:
        img = np.where(img > 0, rng.integers(1, 4, shape), 0).astype(np.uint8)
    if seed % 6 == 5:
        img[0] = 0  # lines along axis 0 starting and ending on zeros (smallest correctors)
        img[-1] = 0
    per = [(True, True, True), (False, False, False), (True, False, True)][seed % 3]
    res = [(1.0, 1.0, 1.0), (0.5, 0.5, 0.5), (1 / 64, 1 / 64, 1 / 64), (0.3, 0.3, 0.3)][seed % 4]
    for squared in (True, False):
        got = D.edt3d(img, periodic=per, resolution=res, squared=squared)
        want = O.edt3d(img, periodic=per, resolution=res, squared=squared)
        np.testing.assert_array_equal(got, want)


def test_edt_subdomain_golden(D, golden, golden_meta):
    from tests._helpers import geom_from_meta
    for ci, case in enumerate(golden_meta["sub_cases"]):
        g = geom_from_meta(O, case["geom"])
        sd = _FakeSD(g)
        np.testing.assert_array_equal(D.edt(golden[f"sub_{ci}_img"], sd), golden[f"sub_{ci}_edt"])


class _FakeDomain:
    def __init__(self, g):
        self.resolution = g.resolution
        self.periodic = g.periodic
        self.boundary_types = g.boundary_types
        self.num_subdomains = 1


class _FakeSD:
    def __init__(self, g):
        self.domain = _FakeDomain(g)
        self.pad = g.pad


def test_c1_full_size_hashes(D, golden_meta):
    """128^3 periodic pack (400 spheres): EDT digests equal the reference's."""
    for seed, want in golden_meta["c1_full"].items():
        r2 = np.random.default_rng(int(seed))
        sph = np.c_[r2.random((400, 3)), r2.uniform(0.03, 0.08, 400)]
        g = O.Geom((128, 128, 128), boundary_types=(("periodic",) * 2,) * 3)
        img = O.gen_pm_spheres_domain(g, sph)
        assert hashlib.sha256(img.tobytes()).hexdigest() == want["img_sha"]
        own = np.ascontiguousarray(img[1:-1, 1:-1, 1:-1])
        e3 = D.edt3d(own, periodic=(True, True, True))
        assert hashlib.sha256(e3.tobytes()).hexdigest() == want["edt3d_sha"]
        es = D.edt(img, _FakeSD(g))
        assert hashlib.sha256(es.tobytes()).hexdigest() == want["edt_sd_sha"]
