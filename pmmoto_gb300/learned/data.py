"""Training data of the schedule network: exact drainage curves on Gaussian
random field media.

A medium is an n^3 GRF (``domain_generation.grf``: hash noise, binomial
smoothing of sigma voxels, pore where the field is at or below its porosity
quantile) placed in the drainage geometry of the plain-drainage
configuration: walls on the y and z faces (one-voxel solid halo), inlet at
x-, outlet at x+, voxel size 1/n.  Its curve is the exact drainage
(``equilibrium_distribution.drainage_counts``, mode "distance", standard
method) at the 64 radii r_k = r_max (k + 1) / 64, k = 0..63, r_max the
medium's largest distance, swept from the largest radius down (capillary
pressures ascending); S[k] is the wetting saturation after radius r_k.
The network input is the medium's distance field (the one its max distance
comes from) averaged to 64^3 and divided by r_max.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _dev
from .._lib import check, host_ptr, i64_array
from ..core.geometry import geo_of
from ..domain_generation import grf
from . import net as netmod

N_RADII = 64


def drainage_kwargs():
    return dict(boundary_types=(("end", "end"), ("wall", "wall"), ("wall", "wall")),
                inlet=((True, False), (False, False), (False, False)),
                outlet=((False, True), (False, False), (False, False)))


def radii_grid(r_max: float) -> np.ndarray:
    """The 64 probe radii (domain units), ascending."""
    return r_max * (np.arange(N_RADII) + 1.0) / N_RADII


def padded_medium(own: torch.Tensor) -> torch.Tensor:
    """Pore image of the drainage geometry from an own-region medium (x has no
    halo: END faces; y and z get a solid one-voxel wall halo)."""
    n0, n1, n2 = own.shape
    img = torch.zeros((n0, n1 + 2, n2 + 2), dtype=torch.uint8, device=own.device)
    img[:, 1:-1, 1:-1] = own
    return img


def grf_batch(n: int, seeds, sigma: float, porosity) -> torch.Tensor:
    """Own-region GRF media [len(seeds), n, n, n] (uint8) of one sigma (each
    the medium gen_grf_medium(n, porosity, seed, sigma=sigma) gives)."""
    f = torch.stack([grf.noise((n, n, n), int(s)) for s in seeds])
    f = grf.smooth_device(f, grf.order_for_sigma(sigma))
    return grf.threshold(f, porosity)


def features(sd, pm) -> torch.Tensor:
    """Network input of a medium: bf16 [64, 64, 64], the own region's distance
    field averaged over 64^3 cells, divided by the max distance."""
    g = geo_of(sd)
    d = pm.distance
    d = d if isinstance(d, torch.Tensor) else torch.as_tensor(np.ascontiguousarray(d), device="cuda")
    out = torch.empty((64, 64, 64), dtype=torch.bfloat16, device=d.device)
    box = np.ascontiguousarray([v for lohi in g.own_box() for v in lohi], dtype=np.int64)
    check(netmod.L().pmg_cnn_downsample(_dev.ptr(d), host_ptr(i64_array(d.shape)), host_ptr(box),
                                        float(pm.max_distance), ctypes.c_void_p(out.data_ptr()),
                                        _dev.stream_ptr(d.device)), "cnn downsample")
    return out


def curve_at(sd, pm, radius_idx, r_max: float):
    """Exact saturations after the radii of radius_idx (indices into the
    64-radius grid), swept from the largest radius down with the multiphase
    image carried from one to the next: {k: S}."""
    from ..domain_generation import Multiphase
    from ..filters import equilibrium_distribution as ED

    grid = radii_grid(r_max)
    order = sorted(set(int(k) for k in radius_idx), reverse=True)
    mp = Multiphase(pm, _mp_constant(pm), 2)
    counts, _ = ED.drainage_counts(mp, [float(grid[k]) for k in order], mode="distance")
    total = float(np.prod(sd.domain.voxels))
    phi = pm.porosity
    return {k: float(c / total) / phi for k, c in zip(order, counts)}


def _mp_constant(pm):
    img = pm.img if isinstance(pm.img, torch.Tensor) else torch.as_tensor(pm.img, device="cuda")
    return torch.where(img == 1, 2, 0).to(torch.uint8)


def dense_curve(sd, pm) -> np.ndarray:
    """S[k] for all 64 radii (ascending radius)."""
    r_max = float(pm.max_distance)
    s = curve_at(sd, pm, range(N_RADII), r_max)
    return np.array([s[k] for k in range(N_RADII)])


def make_examples(count: int, seed: int = 0, sizes=(96, 128, 160), sigmas=(2.5, 3.0, 3.5, 4.0, 5.0, 6.0),
                  porosity=(0.3, 0.6), batch: int = 32, workers: int = 8, log=None):
    """`count` (input, curve) pairs on the device: X bf16 [count, 64^3], Y fp32
    [count, 64], plus the media parameters.  Media are generated `batch` at a
    time (one sigma and size per batch) and their curves computed
    concurrently on `workers` CUDA streams (pmmoto_gb300.batch)."""
    import time

    import pmmoto_gb300 as P
    from .. import batch as B

    rng = np.random.default_rng(seed)
    tm = {"grf": 0.0, "curves": 0.0}
    X = torch.empty((count, 64 ** 3), dtype=torch.bfloat16, device="cuda")
    Y = torch.empty((count, N_RADII), dtype=torch.float32, device="cuda")
    meta = []
    i = 0
    while i < count:
        n = int(rng.choice(sizes))
        sigma = float(rng.choice(sigmas))
        b = min(batch, count - i)
        seeds = rng.integers(1, 2 ** 31, b)
        por = rng.uniform(*porosity, b)
        t0 = time.perf_counter()
        media = grf_batch(n, seeds, sigma, por)
        torch.cuda.synchronize()
        t1 = time.perf_counter()

        def one(j):
            sd = P.initialize((n,) * 3, box=((0.0, 1.0),) * 3, **drainage_kwargs())
            pm = P.domain_generation.PorousMedia(sd, padded_medium(media[j]))
            if pm.max_distance <= 0:
                return None
            y = dense_curve(sd, pm)
            x = features(sd, pm).reshape(-1).clone()
            return x, y, (n, sigma, float(por[j]), int(seeds[j]), float(pm.max_distance) * n)

        for r in B.map_streams(one, range(b), workers=workers):
            if r is None or i >= count:
                continue
            X[i] = r[0]
            Y[i] = torch.as_tensor(r[1], dtype=torch.float32)
            meta.append(r[2])
            i += 1
        torch.cuda.synchronize()
        tm["grf"] += t1 - t0
        tm["curves"] += time.perf_counter() - t1
        if log:
            log(i)
    make_examples.timing = tm
    return X, Y, meta
