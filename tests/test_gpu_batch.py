"""Concurrent media on CUDA streams give exactly the sequential results."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _packs(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        vox = tuple(int(v) for v in rng.choice([24, 32, 40], 3))
        box = [v / 32.0 for v in vox]
        n = int(rng.integers(20, 60))
        sph = np.empty((n, 4))
        for d in range(3):
            sph[:, d] = rng.random(n) * box[d]
        sph[:, 3] = rng.uniform(0.05, 0.15, n)
        out.append((vox, box, sph))
    return out


def test_drainage_batch_matches_sequential():
    import torch

    import pmmoto_gb300 as P
    from pmmoto_gb300 import batch
    from pmmoto_gb300.filters import equilibrium_distribution as ED

    bts = (("end", "end"), ("wall", "wall"), ("wall", "wall"))
    inlet = ((True, False), (False, False), (False, False))
    outlet = ((False, True), (False, False), (False, False))
    pcs = sorted(2.0 / (np.linspace(1, 4, 6) / 32.0))

    def make(vox, box, sph):
        sd = P.initialize(vox, box=tuple((0.0, b) for b in box), boundary_types=bts, inlet=inlet, outlet=outlet)
        pm = P.domain_generation.gen_pm_spheres_domain(sd, torch.as_tensor(sph, device="cuda"))
        return P.domain_generation.gen_mp_constant(pm, 2)

    packs = _packs(6, 3)
    seq = [ED.drainage(make(*p), pcs, mode="distance") for p in packs]
    par = batch.drainage_batch([make(*p) for p in packs], pcs, workers=3, mode="distance")
    for a, b in zip(seq, par):
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


def test_map_streams_order():
    from pmmoto_gb300 import batch

    assert batch.map_streams(lambda x: x * x, list(range(10)), workers=4) == [x * x for x in range(10)]
