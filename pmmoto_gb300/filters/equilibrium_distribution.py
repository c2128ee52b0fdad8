"""Drop-in for ``pmmoto.filters.equilibrium_distribution`` on the GPU
(src/pmmoto/filters/equilibrium_distribution.py:25-289).

The standard (Hilpert & Miller) drainage runs on the device in one native
call: for every capillary pressure the probe radius is formed on the host
exactly as the reference forms it (float64), and the porosimetry step, the
outlet-connected wetting phase, the update and the saturation count run as
CUDA kernels without host round trips beyond porosimetry's branch tests.
"""

from __future__ import annotations

import logging

import numpy as np
import torch

from .. import _dev
from .._lib import check, host_ptr, i64_array, lib
from ..core.geometry import geo_of
from . import morphological_operators as morph
from .porosimetry import MODES

__all__ = ["drainage"]


def _radius(pc, gamma, contact_angle):
    """Multiphase.get_probe_radius (multiphase.py:98-116)."""
    if pc == 0:
        return 0
    return 2.0 * gamma / pc * np.cos(np.deg2rad(contact_angle))


def _inactive(multiphase, r, rd):
    """The reference's empty-morph rule (equilibrium_distribution.py:158-166,
    :206-214, :262-270): a radius below the finest resolution or above the
    medium's largest distance."""
    return min(r, rd) < min(multiphase.subdomain.domain.resolution) or max(r, rd) > \
        multiphase.porous_media.max_distance


def drainage_counts(multiphase, radii, mode="distance", radii_dilate=None, start=None):
    """Run the drainage sweep for the given probe radii on the device; returns
    (per-radius own-region phase-2 counts, final multiphase CUDA tensor).
    radii_dilate: dilation radii when they differ from the erosion radii
    (extended contact-angle method); start: the multiphase image to start
    from (default multiphase.img)."""
    sd = multiphase.subdomain
    g = geo_of(sd)
    pm, _ = morph.to_u8(multiphase.porous_media.img)
    mp, _ = morph.to_u8(multiphase.img if start is None else start)
    mp = mp.clone()
    n = len(radii)
    if radii_dilate is None:
        radii_dilate = radii
    active = np.zeros(n, dtype=np.int32)
    ratios = np.zeros((max(n, 1), 3), dtype=np.int32)
    ratios_d = np.zeros((max(n, 1), 3), dtype=np.int32)
    rad = np.zeros(max(n, 1), dtype=np.float64)
    rad_d = np.zeros(max(n, 1), dtype=np.float64)
    be = np.full(max(n, 1), -1.0)
    bd = np.full(max(n, 1), -1.0)
    for k, (r, rd) in enumerate(zip(radii, radii_dilate)):
        rad[k] = float(r)
        rad_d[k] = float(rd)
        if _inactive(multiphase, r, rd):
            continue
        morph.check_radii(sd, [r, rd])
        active[k] = 1
        ratios[k] = morph.element_ratio(g.res, r)
        ratios_d[k] = morph.element_ratio(g.res, rd)
        if mode == "morph":
            be[k] = morph.ball_sq(g.res, r)
        if mode in ("morph", "hybrid"):
            bd[k] = morph.ball_sq(g.res, rd)
    from .connected_components import _box

    counts = np.zeros(max(n, 1), dtype=np.int64)
    rpad = np.ascontiguousarray([g.rpad[d][s] for d in range(3) for s in (0, 1)], dtype=np.int32)
    res32 = np.ascontiguousarray([np.float32(r) for r in g.res], dtype=np.float32)
    own = np.ascontiguousarray([v for lohi in g.own_box() for v in lohi], dtype=np.int64)
    st = lib().pmg_drainage_ext(_dev.ptr(pm), _dev.ptr(mp), host_ptr(i64_array(pm.shape)), host_ptr(g.bc_codes()),
                                host_ptr(g.pad_flat()), host_ptr(rpad), host_ptr(own),
                                host_ptr(_box(g.face_slab("inlet"))), host_ptr(_box(g.face_slab("outlet"))),
                                host_ptr(res32), n, host_ptr(rad), host_ptr(active), host_ptr(ratios), host_ptr(be),
                                host_ptr(bd), host_ptr(counts), host_ptr(rad_d), host_ptr(ratios_d),
                                _dev.stream_ptr(pm.device))
    check(st, "drainage")
    return counts[:n], mp


def _drainage_saving(multiphase, capillary_pressures, radii, radii_d, mode, out_folder):
    """drainage(save=True) (equilibrium_distribution.py:93-121): the sweep one
    pressure at a time, writing after each update the multiphase image with
    that pressure's morph image to
    <out_folder>/capillary_pressure_<pc with 3 decimals, '.' -> '_'>.vti."""
    from ..io.output import save_img
    from .porosimetry import porosimetry_device

    g = geo_of(multiphase.subdomain)
    pm, _ = morph.to_u8(multiphase.porous_media.img)
    mp, _ = morph.to_u8(multiphase.img)
    counts = np.zeros(len(radii), dtype=np.int64)
    for k, pc in enumerate(capillary_pressures):
        r = radii[k]
        rd = r if radii_d is None else radii_d[k]
        if _inactive(multiphase, r, rd):
            m = torch.zeros_like(pm)
        else:
            m = porosimetry_device(g, pm, r, rd, True, mp, mode)
        c, mp = drainage_counts(multiphase, [r], mode, None if radii_d is None else [rd], start=mp)
        counts[k] = c[0]
        file_out = out_folder + (f"/capillary_pressure_{pc:.3f}".replace(".", "_"))
        save_img(file_out, multiphase.subdomain, mp, additional_img={"morph": m})
    return counts, mp


def drainage(multiphase, capillary_pressures, gamma=1, contact_angle=0, method="standard", mode="hybrid",
             save=False, out_folder="drainage_out"):
    """Wetting-phase saturation at each capillary pressure
    (equilibrium_distribution.py:25-289: standard, contact_angle and
    extended_contact_angle methods).  multiphase.img is updated."""
    if isinstance(capillary_pressures, (int, float)):
        capillary_pressures = [capillary_pressures]
    elif isinstance(capillary_pressures, list):
        sorted_cp = sorted(capillary_pressures)
        if capillary_pressures != sorted_cp:
            logging.warning("The capillary pressure must be monotonically increasing. Sorting.")
            capillary_pressures = sorted_cp
    if method == "standard":
        if contact_angle != 0:
            raise ValueError("The standard approach requires a zero contact angle!")
    elif method in ("contact_angle", "extended_contact_angle"):
        if contact_angle == 0:
            logging.warning("The contact angle is zero. This will yield same results as the standard approach.")
    else:
        raise ValueError(f"{method} is not implemented. ")
    if mode not in MODES:
        raise ValueError(f"mode {mode} must be one of {MODES}")
    # probe radii as Multiphase.get_probe_radius forms them (float64); the
    # extended method (Schulz and Wargo, :230-289) dilates by r |cos(theta)|
    radii = [_radius(pc, gamma, contact_angle) for pc in capillary_pressures]
    radii_d = None
    if method == "extended_contact_angle":
        radii_d = [r * np.abs(np.cos(np.deg2rad(contact_angle))) for r in radii]
    if save:
        counts, mp = _drainage_saving(multiphase, capillary_pressures, radii, radii_d, mode, out_folder)
    else:
        counts, mp = drainage_counts(multiphase, radii, mode, radii_d)
    total = np.prod(multiphase.subdomain.domain.voxels)
    phi = multiphase.porous_media.porosity
    sat = np.zeros(len(capillary_pressures))
    for k in range(len(capillary_pressures)):
        sat[k] = float(counts[k] / total) / phi
    multiphase.img = mp if isinstance(multiphase.img, torch.Tensor) else mp.cpu().numpy()
    return sat
