"""ORACLE -- test infrastructure only.

CPU restatement of PMMoTo's voxel-morphology hot path (EDT, dilate/erode,
connected components with periodic merge, inlet/outlet selection,
porosimetry, drainage, sphere voxelisation), used only by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` as the
checker.  The shipped package never imports this module.

The per-line arithmetic lives in ``pmg_oracle.c`` / ``pmg_oracle_cc.cpp``
(built into ``oracle/_ref/liboracle.so`` by ``oracle/build.py``); this file
restates the reference's Python drivers around it.  Every function cites the
reference routine it follows (paths relative to the PMMoTo v1.0.7 tree).

Geometry is described by :class:`Geom`, a restatement of the single-rank
subdomain metadata (``src/pmmoto/core/subdomain_padded.py``,
``subdomain.py``, ``features.py``, ``domain_decompose.py:62-100``) kept
independent of the package so that the checker does not share code with the
thing it checks.
"""

from __future__ import annotations

import ctypes
import itertools
import math
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "liboracle.so")
_lib = None

END, WALL, PERIODIC = "end", "wall", "periodic"


class OrAxisCfg(ctypes.Structure):
    _fields_ = [
        (n, ctypes.c_int32)
        for n in ("periodic", "f_lo", "l_lo", "l_hi", "a_u", "a_l", "hf_lo", "hb_hi")
    ]


class OrHull(ctypes.Structure):
    _fields_ = [("vertex", ctypes.c_int32), ("height", ctypes.c_float), ("range", ctypes.c_float)]


def lib():
    """Load (building if needed) the oracle's C library."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            from . import build as _build  # noqa: WPS433

            _build.build_oracle()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        L.or_edt3d_sq.argtypes = [P, P, P, P, P, ctypes.c_int]
        L.or_edt2d_sq.argtypes = [P, P, P, P, P, ctypes.c_int]
        L.or_edt_pass0_line.argtypes = [P, P, ctypes.c_int, ctypes.c_long, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_float]
        L.or_parabolic_line.argtypes = [P, ctypes.c_int, ctypes.c_float, ctypes.c_long,
                                        P, ctypes.c_int, P, ctypes.c_int]
        L.or_boundary_hull.argtypes = [P, ctypes.c_int, ctypes.c_float, ctypes.c_long,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.or_boundary_hull.restype = ctypes.c_int
        L.or_spheres.argtypes = [P, ctypes.c_long, P, P, P, P, P]
        L.or_cc_label.argtypes = [P, ctypes.c_int, P, P]
        L.or_cc_label.restype = ctypes.c_int64
        L.or_unique_pairs.argtypes = [P, ctypes.c_int64, P]
        L.or_unique_pairs.restype = ctypes.c_int64
        _lib = L
    return _lib


class _Ptr(ctypes.c_void_p):
    """c_void_p that keeps its array alive for the duration of the call."""


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    p = _Ptr(a.ctypes.data)
    p._keep = a
    return p


# --------------------------------------------------------------------------
# 1-D kernels (test hooks of _distance.pyx:219-237, 401-454, 679-702)
# --------------------------------------------------------------------------

def initial_envelope_1d(img, lower_corrector=np.inf, upper_corrector=np.inf, resolution=1.0):
    """squared_edt_1d on one line (determine_initial_envelope_1d)."""
    img = np.ascontiguousarray(img, dtype=np.uint8)
    out = np.zeros(img.shape[0], dtype=np.float32)
    lib().or_edt_pass0_line(_ptr(img), _ptr(out), img.shape[0], 1, float(np.float32(resolution)),
                            float(np.float32(lower_corrector)), float(np.float32(upper_corrector)))
    return out


def _hulls_to_c(hulls):
    arr = (OrHull * max(1, len(hulls)))()
    for i, h in enumerate(hulls):
        arr[i].vertex = int(h["vertex"])
        arr[i].height = float(h["height"])
        arr[i].range = float(h["range"])
    return arr


def parabolic_envelope_1d(img, resolution=1.0, lower_hull=(), upper_hull=()):
    """squared_edt_1d_parabolic on one line (determine_parabolic_envelope_1d)."""
    out = np.array(img, dtype=np.float32, copy=True)
    lo, up = _hulls_to_c(list(lower_hull)), _hulls_to_c(list(upper_hull))
    lib().or_parabolic_line(_ptr(out), out.shape[0], float(np.float32(resolution)), 1,
                            ctypes.addressof(lo), len(lower_hull), ctypes.addressof(up), len(upper_hull))
    return out


def boundary_hull_1d(img, start, end, resolution=1.0, num_hull=4, forward=True):
    """return_boundary_hull on one line (get_boundary_hull_1d, _distance.pyx:679-702)."""
    work = np.array(img, dtype=np.float32, copy=True)
    out = (OrHull * (num_hull + 2))()
    seg = work[start:]
    c = lib().or_boundary_hull(_ptr(seg), int(end), float(np.float32(resolution)), 1,
                               int(num_hull), int(start), 1 if forward else 0,
                               ctypes.addressof(out))
    return [{"vertex": out[i].vertex, "height": out[i].height, "range": out[i].range}
            for i in range(c)]


# --------------------------------------------------------------------------
# EDT drivers
# --------------------------------------------------------------------------

def _edt3d_cfg(periodic):
    return (OrAxisCfg * 3)(*[OrAxisCfg(int(bool(p)), 0, 0, 0, 1, 0, 0, 0) for p in periodic])


def _run_edt3d(img, res32, cfg, num_hull=4):
    img = np.ascontiguousarray(img)
    if img.dtype == np.bool_:
        img = img.view(np.uint8)
    img = np.ascontiguousarray(img, dtype=np.uint8)
    out = np.empty(img.shape, dtype=np.float32)
    shape = np.array(img.shape, dtype=np.int64)
    res = np.array(res32, dtype=np.float32)
    lib().or_edt3d_sq(_ptr(img), _ptr(out), _ptr(shape), _ptr(res), ctypes.addressof(cfg), num_hull)
    return out


def edt3d(img, periodic=(False, False, False), resolution=(1.0, 1.0, 1.0), squared=False, num_hull=4):
    """edt3d, euclidean_distance_transform.py:208-303."""
    out = _run_edt3d(img, [np.float32(r) for r in resolution], _edt3d_cfg(periodic), num_hull)
    return out if squared else np.sqrt(out)


def edt2d(img, periodic=(False, False), resolution=(1.0, 1.0), num_hull=4):
    """edt2d, euclidean_distance_transform.py:104-205."""
    img = np.ascontiguousarray(img, dtype=np.uint8)
    out = np.empty(img.shape, dtype=np.float32)
    shape = np.array(img.shape, dtype=np.int64)
    res = np.array([np.float32(r) for r in resolution], dtype=np.float32)
    per = np.array([int(bool(p)) for p in periodic], dtype=np.int32)
    lib().or_edt2d_sq(_ptr(img), _ptr(out), _ptr(shape), _ptr(res), _ptr(per), num_hull)
    return np.sqrt(out)


def corrected_edt_sq(img, geom: "Geom", num_hull=4):
    """corrected_edt (euclidean_distance_transform.py:56-101) on one rank, squared.

    Axis 0 correctors: get_nearest_boundary_distance (:306-392) with
    which_voxels="pad", distance_to="own"; the x+ face inherits the lower skip
    set by the x- face because the skip variables are not reset between faces.
    Axes 1-2: get_boundary_hull (:450-528) with skips 2*pad.
    """
    cfgs = []
    for d in range(3):
        plo, phi = geom.pad[d]
        per = geom.axis_periodic(d)
        cfgs.append(OrAxisCfg(int(per), 2 * plo, 2 * plo, 2 * phi, -plo, -phi - 1, 2 * plo, 2 * phi))
    cfg = (OrAxisCfg * 3)(*cfgs)
    return _run_edt3d(img, [np.float32(r) for r in geom.resolution], cfg, num_hull)


def edt(img, geom: "Geom | None" = None):
    """edt, euclidean_distance_transform.py:25-53 (single rank)."""
    if geom is not None:
        if geom.periodic:
            return np.sqrt(corrected_edt_sq(img, geom))
        return edt3d(img, resolution=geom.resolution)
    if img.ndim == 3:
        return edt3d(img)
    if img.ndim == 2:
        return edt2d(img)
    raise ValueError(f"Wrong img dimension {img.shape}")


# --------------------------------------------------------------------------
# Single-rank geometry
# --------------------------------------------------------------------------

FACES = [d for d in itertools.product(*[[-1, 0, 1]] * 3) if sum(abs(x) for x in d) == 1]
EDGES = [d for d in itertools.product([-1, 0, 1], repeat=3) if sum(abs(x) for x in d) == 2]
CORNERS = [(x, y, z) for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)]
ALL_FEATURES = FACES + EDGES + CORNERS  # orientation.py:40-183 iteration order


@dataclass
class Geom:
    """Single-rank padded subdomain (pmmoto.initialize with subdomains=(1,1,1))."""

    voxels: tuple  # domain (own) voxels
    boundary_types: tuple = ((END, END), (END, END), (END, END))
    box: tuple = ((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))
    inlet: tuple = ((False, False), (False, False), (False, False))
    outlet: tuple = ((False, False), (False, False), (False, False))
    reservoir_voxels: int = 0
    pad_in: tuple = (1, 1, 1)
    resolution: tuple = field(init=False)
    pad: tuple = field(init=False)
    reservoir_pad: tuple = field(init=False)
    shape: tuple = field(init=False)

    def __post_init__(self):
        self.boundary_types = tuple(tuple(str(getattr(b, "value", b)) for b in bt) for bt in self.boundary_types)
        length = [float(b[1]) - float(b[0]) for b in self.box]
        self.resolution = tuple(length[d] / self.voxels[d] for d in range(3))
        pad = []
        for d in range(3):
            lo, hi = self.boundary_types[d]
            pad.append((0 if lo == END else 1 if lo == WALL else self.pad_in[d],
                        0 if hi == END else 1 if hi == WALL else self.pad_in[d]))
        self.pad = tuple(pad)
        self.sd_inlet = tuple((bool(self.inlet[d][0]) and self.boundary_types[d][0] == END,
                               bool(self.inlet[d][1]) and self.boundary_types[d][1] == END) for d in range(3))
        self.sd_outlet = tuple((bool(self.outlet[d][0]) and self.boundary_types[d][0] == END,
                                bool(self.outlet[d][1]) and self.boundary_types[d][1] == END) for d in range(3))
        if self.reservoir_voxels:
            self.reservoir_pad = tuple((self.reservoir_voxels if self.sd_inlet[d][0] else 0,
                                        self.reservoir_voxels if self.sd_inlet[d][1] else 0) for d in range(3))
        else:
            self.reservoir_pad = ((0, 0), (0, 0), (0, 0))
        self.shape = tuple(self.voxels[d] + sum(self.pad[d]) + sum(self.reservoir_pad[d]) for d in range(3))

    @property
    def periodic(self):
        return any(b == PERIODIC for bt in self.boundary_types for b in bt)

    def axis_periodic(self, d):
        return self.boundary_types[d][0] == PERIODIC

    def coords(self):
        """get_padded_box + get_coords (subdomain_padded.py:188-216, domain_discretization.py:70-90)."""
        out = []
        for d in range(3):
            res = self.resolution[d]
            length = self.voxels[d] * res
            lower = self.box[d][1] - length
            upper = lower + length
            lower = lower - (self.pad[d][0] + self.reservoir_pad[d][0]) * res
            upper = upper + (self.pad[d][1] + self.reservoir_pad[d][1]) * res
            half = 0.5 * res
            out.append(np.linspace(lower + half, upper - half, self.shape[d]))
        return out

    def own_slices(self):
        """get_own_voxels, subdomain_padded.py:271-283."""
        return tuple(slice(self.pad[d][0] + self.reservoir_pad[d][0],
                           self.shape[d] - self.pad[d][1] - self.reservoir_pad[d][1]) for d in range(3))

    # features.py:76-139 and subdomain_features.py:105-158 ---------------
    def feature_btype(self, f):
        types = []
        for d in range(3):
            if f[d] == -1:
                types.append(self.boundary_types[d][0])
            elif f[d] == 1:
                types.append(self.boundary_types[d][1])
        if END in types:
            return END
        if WALL in types:
            return WALL
        return PERIODIC

    def feature_has_neighbor(self, f):
        """domain_decompose.py:62-100 on one rank: only all-periodic features wrap to rank 0."""
        return all(f[d] == 0 or self.boundary_types[d][0] == PERIODIC for d in range(3))

    def feature_slabs(self, f, shape=None, pad=None):
        shape = self.shape if shape is None else shape
        pad = self.pad if pad is None else pad
        bt = self.feature_btype(f)
        padded = any(p for pp in pad for p in pp)
        own, nb = [], []
        for d in range(3):
            length = shape[d]
            pb, pa = pad[d]
            if f[d] == -1:
                if pb and bt != WALL:
                    own.append((pb, 2 * pb))
                elif pb and bt == WALL:
                    own.append((1, 2))
                else:
                    own.append((0, 1))
                nb.append(((0, 1) if bt == WALL else (0, pb)) if padded else (0, 0))
            elif f[d] == 1:
                if pa and bt != WALL:
                    own.append((length - 2 * pa, length - pa))
                elif pa and bt == WALL:
                    own.append((length - 2, length - 1))
                else:
                    own.append((length - 1, length))
                nb.append(((length - 1, length) if bt == WALL else (length - pa, length)) if padded else (0, 0))
            else:
                own.append((pb, length - pa))
                nb.append((pb, length - pa) if padded else (0, 0))
        return tuple(slice(a, b) for a, b in own), tuple(slice(a, b) for a, b in nb)

    def set_wall_bcs(self, img):
        """set_wall_bcs, subdomain.py:273-287."""
        for f in FACES:
            if self.feature_btype(f) == WALL:
                sl = [slice(None)] * 3
                d = [i for i in range(3) if f[i] != 0][0]
                sl[d] = 0 if f[d] == -1 else -1
                img[tuple(sl)] = 0
        return img

    def update_reservoir(self, img, value):
        """update_reservoir, subdomain_padded.py:285-307."""
        for d, (a, b) in enumerate(self.reservoir_pad):
            if a > 0:
                sl = [slice(None)] * 3
                sl[d] = slice(0, a)
                img[tuple(sl)] = value
            if b > 0:
                sl = [slice(None)] * 3
                sl[d] = slice(-b, None)
                img[tuple(sl)] = value
        return img


def _opp(f):
    return tuple(-x for x in f)


def update_buffer(geom: Geom, img):
    """update_buffer (communication.py:101-118, 160-228) on one rank."""
    send = {}
    for f in ALL_FEATURES:
        if geom.feature_has_neighbor(f):
            own, _ = geom.feature_slabs(f)
            send[f] = img[own]
    out = img.copy()
    for f in ALL_FEATURES:
        if geom.feature_has_neighbor(f) and _opp(f) in send:
            _, nb = geom.feature_slabs(f)
            out[nb] = send[_opp(f)]
    return geom.set_wall_bcs(out)


def update_extended_buffer(geom: Geom, img, buffer):
    """update_extended_buffer (communication.py:121-157), extend_padding (subdomain_padded.py:116-167)."""
    if any(geom.voxels[d] < buffer[d] for d in range(3)):
        raise SystemExit(1)
    ext = []
    for d in range(3):
        lo, hi = geom.boundary_types[d]
        elo = 0 if lo == END or (lo == WALL and geom.pad[d][0] == 1) else buffer[d]
        ehi = 0 if hi == END or (hi == WALL and geom.pad[d][1] == 1) else buffer[d]
        ext.append((elo, ehi))
    total_pad = tuple((geom.pad[d][0] + ext[d][0], geom.pad[d][1] + ext[d][1]) for d in range(3))
    shape = tuple(geom.shape[d] + ext[d][0] + ext[d][1] for d in range(3))
    _img = np.pad(img.copy(), ext, "constant", constant_values=255)
    send = {}
    for f in ALL_FEATURES:
        if geom.feature_has_neighbor(f):
            own, _ = geom.feature_slabs(f, shape, total_pad)
            send[f] = _img[own]
    out = _img.copy()
    for f in ALL_FEATURES:
        if geom.feature_has_neighbor(f) and _opp(f) in send:
            _, nb = geom.feature_slabs(f, shape, total_pad)
            out[nb] = send[_opp(f)]
    out = geom.set_wall_bcs(out)
    assert not np.any(out == 255)
    return out, tuple(ext)


def _unpad(img, pad):
    return np.ascontiguousarray(img[tuple(slice(p[0], img.shape[i] - p[1]) for i, p in enumerate(pad))])


def struct_ratio(resolution, radius):
    """gen_struct_ratio + the isotropy check of gen_struct_element (morphological_operators.py:35-100)."""
    if resolution[0] != resolution[1] != resolution[2]:
        raise ValueError("Resolution must be isotropic for morphological methods.")
    if radius < np.min(resolution):
        raise ValueError(f"The chosen radius {radius} is too small! The resolutions is {resolution}")
    return tuple(int(math.ceil(radius / res)) for res in resolution)


def struct_element(resolution, radius):
    """gen_struct_element, morphological_operators.py:66-100."""
    ratio = struct_ratio(resolution, radius)
    grids = [np.linspace(-r, r, r * 2 + 1) for r in ratio]
    xg, yg, zg = np.meshgrid(*grids, indexing="ij")
    s = xg**2 + yg**2 + zg**2
    r = radius / resolution[0]
    return ratio, np.array(s <= r * r, dtype=np.uint8)


def addition(geom: Geom, img, radius, fft=False):
    """addition, morphological_operators.py:103-149."""
    ratio, se = struct_element(geom.resolution, radius)
    halo_img, halo = update_extended_buffer(geom, img, ratio)
    if fft:
        from scipy.signal import fftconvolve

        out = (fftconvolve(halo_img, se, mode="same") > 0.1).astype(np.uint8)
    else:
        d = edt3d(np.logical_not(halo_img), resolution=geom.resolution)
        out = np.where((d <= radius), 1, 0).astype(np.uint8)
    out = _unpad(out, halo)
    return geom.set_wall_bcs(out)


def subtraction(geom: Geom, img, radius, fft=False):
    """subtraction, morphological_operators.py:175-228."""
    ratio, se = struct_element(geom.resolution, radius)
    halo_img, halo = update_extended_buffer(geom, img, ratio)
    if fft:
        from scipy.signal import fftconvolve

        _pad = 1
        if any(b == END for bt in geom.boundary_types for b in bt):
            _pad = int(np.max(ratio))
        _img = np.pad(halo_img, _pad, mode="constant", constant_values=1)
        _img = fftconvolve(_img, se, mode="same") > (se.sum() - 0.1)
        out = _unpad(_img, tuple((_pad, _pad) for _ in range(3))).astype(np.uint8)
    else:
        d = edt3d(halo_img, resolution=geom.resolution)
        out = np.where((d <= radius), 0, 1).astype(np.uint8)
    out = _unpad(out, halo)
    return geom.set_wall_bcs(out)


dilate = addition
erode = subtraction


def opening(geom, img, radius):
    return addition(geom, subtraction(geom, img, radius), radius)


def closing(geom, img, radius):
    return subtraction(geom, addition(geom, img, radius), radius)


# --------------------------------------------------------------------------
# Connected components
# --------------------------------------------------------------------------

def cc_label(img):
    """cc3d.connected_components(img, return_N=True, out_dtype=uint64): see pmg_oracle_cc.cpp."""
    img = np.ascontiguousarray(img)
    if img.dtype == np.bool_:
        img = img.view(np.uint8)
    if img.dtype.itemsize not in (1, 2, 4, 8):
        raise ValueError("unsupported dtype")
    labels = np.zeros(img.shape, dtype=np.uint64)
    shape = np.array(img.shape, dtype=np.int64)
    n = lib().or_cc_label(_ptr(img), img.dtype.itemsize, _ptr(labels), _ptr(shape))
    return labels, int(n)


def unique_pairs(pairs):
    pairs = np.ascontiguousarray(pairs, dtype=np.uint64)
    out = np.zeros_like(pairs)
    m = lib().or_unique_pairs(_ptr(pairs), pairs.shape[0], _ptr(out))
    return out[:m]


def connect_components(img, geom: Geom):
    """connect_components + connect_subdomain_boundaries (connected_components.py:32-101),
    voxels.py:167-397, _voxels.pyx:335-383 and :548-579, on one rank."""
    labels, count = cc_label(img)
    if not geom.periodic:
        return labels, count
    boundary = {}
    for f in ALL_FEATURES:
        if not geom.feature_has_neighbor(f):
            continue
        own, nb = geom.feature_slabs(f)
        boundary[f] = {"own": labels[own].flatten(), "neighbor": labels[nb].flatten()}
    recv = {f: boundary[_opp(f)] for f in boundary if _opp(f) in boundary}
    matches: dict = {}
    for f in ALL_FEATURES:
        if f not in recv:
            continue
        to_match = np.stack([np.concatenate((boundary[f]["own"], boundary[f]["neighbor"])),
                             np.concatenate((recv[f]["neighbor"], recv[f]["own"]))], axis=1)
        m = unique_pairs(to_match)
        m = m[~np.any(m == 0, axis=1)]
        for a, b in m:
            key, nbr = (0, int(a)), (0, int(b))
            if key not in matches:
                matches[key] = {"neighbor_matches": [nbr]}
            elif nbr not in matches[key]["neighbor_matches"]:
                matches[key]["neighbor_matches"].append(nbr)
    # merge_matched_voxels
    visited = {k: False for k in matches}
    gmap = {}
    global_id = 1
    for key in matches:
        if visited[key]:
            continue
        queue, conns = [key], []
        while queue:
            cur = queue.pop()
            if visited[cur]:
                continue
            visited[cur] = True
            conns.append(cur)
            for nb in matches[cur]["neighbor_matches"]:
                if not visited[nb]:
                    queue.append(nb)
        for c in conns:
            gmap[c] = global_id
        global_id += 1 if conns else 0
    # local_to_global_labeling
    start = global_id
    lut = np.zeros(count + 1, dtype=np.uint64)
    n_local = 0
    for n in range(1, count + 1):
        if (0, n) in gmap:
            lut[n] = gmap[(0, n)]
        else:
            lut[n] = start + n_local
            n_local += 1
    max_label = n_local + start
    if max_label < 1:
        max_label = global_id
    return lut[labels], int(max_label)


def _face_labels(geom: Geom, labels, which):
    """gen_inlet_label_map / gen_outlet_label_map (voxels.py:400-454): the last flagged face wins."""
    flags = geom.sd_inlet if which == "inlet" else geom.sd_outlet
    sel = np.empty(0, dtype=np.uint64)
    for f in FACES:
        d = [i for i in range(3) if f[i] != 0][0]
        side = 0 if f[d] < 0 else 1
        if flags[d][side]:
            own, _ = geom.feature_slabs(f)
            sel = np.unique(labels[own])
    return sel


def _connected_img(geom: Geom, img, phase, keep):
    labels, _ = connect_components(img, geom)
    inl = _face_labels(geom, labels, "inlet")
    outl = _face_labels(geom, labels, "outlet")
    maxl = int(labels.max()) if labels.size else 0
    is_in = np.zeros(maxl + 1, dtype=bool)
    is_out = np.zeros(maxl + 1, dtype=bool)
    is_in[inl[inl > 0].astype(np.int64)] = True
    is_out[outl[outl > 0].astype(np.int64)] = True
    lut = np.zeros(maxl + 1, dtype=np.uint64)
    flat_l = labels.ravel()
    lut[flat_l] = np.asarray(img).ravel().astype(np.uint64)
    ok = keep(is_in, is_out)
    if phase is not None:
        ok &= lut == np.uint64(phase)
    lut = np.where(ok, lut, np.uint64(0))
    return lut[labels]


def inlet_connected_img(geom, img, phase=None):
    """inlet_connected_img, connected_components.py:254-296."""
    return _connected_img(geom, img, phase, lambda i, o: i.copy())


def outlet_connected_img(geom, img, phase=None):
    """outlet_connected_img, connected_components.py:299-341."""
    return _connected_img(geom, img, phase, lambda i, o: o.copy())


def inlet_outlet_connected_img(geom, img, phase=None):
    """inlet_outlet_connected_img, connected_components.py:203-251."""
    return _connected_img(geom, img, phase, lambda i, o: i & o)


def isolated_img(geom, img, phase=None):
    """isolated_img, connected_components.py:344-392."""
    return _connected_img(geom, img, phase, lambda i, o: ~(i | o))


# --------------------------------------------------------------------------
# Porosimetry and drainage
# --------------------------------------------------------------------------

def porosimetry(geom: Geom, pm_img, radius, inlet=False, mp_img=None, mode="distance"):
    """porosimetry, porosimetry.py:84-160."""
    if isinstance(radius, (int, float)):
        r_e = r_d = radius
    elif isinstance(radius, list) and len(radius) == 2:
        r_e, r_d = radius
    else:
        raise ValueError(f"Radius {radius} must either be a number or a list of length 2")
    for r in (r_e, r_d):
        ratio = struct_ratio(geom.resolution, r)
        if any(geom.voxels[d] < ratio[d] for d in range(3)):
            raise SystemExit(1)
    res = subtraction(geom, pm_img, r_e, fft=(mode == "morph"))
    if inlet:
        res = inlet_connected_img(geom, res)
    if np.count_nonzero(res == 1) > 0:
        if mp_img is not None and np.count_nonzero(mp_img == 1) > 0:
            n_conn = inlet_connected_img(geom, mp_img, 1)
            res = np.where((res != 1) | (n_conn != 1), 0, res)
        res = addition(geom, res, r_d, fft=(mode in ("morph", "hybrid")))
    return res.astype(np.uint8)


def porosity(geom: Geom, pm_img):
    """PorousMedia.set_porosity, porousmedia.py:53-66."""
    own = pm_img[geom.own_slices()]
    return np.count_nonzero(own == 1) / np.prod(geom.voxels)


def max_distance(geom: Geom, pm_img):
    """PorousMedia.max_distance (porousmedia.py:82-101): max of edt(img, sd) after a halo update."""
    d = edt(pm_img, geom)
    d = update_buffer(geom, d)
    return float(np.amax(d))


def drainage(geom: Geom, pm_img, capillary_pressures, gamma=1, mode="distance", dmax=None, contact_angle=0,
             method="standard", mp_img=None, phi=None):
    """drainage with _standard_method, _contact_angle_method or
    _extended_contact_angle_method (equilibrium_distribution.py:25-289),
    starting from mp_img (default: gen_mp_constant(pm, 2)).

    Returns (saturations, final multiphase image)."""
    if isinstance(capillary_pressures, (int, float)):
        capillary_pressures = [capillary_pressures]
    elif isinstance(capillary_pressures, list):
        capillary_pressures = sorted(capillary_pressures)
    if mp_img is None:
        mp_img = np.where(pm_img == 1, 2, 0).astype(np.uint8)
    if phi is None:
        phi = porosity(geom, pm_img)
    sat = np.zeros(len(capillary_pressures))
    theta = contact_angle if method != "standard" else 0
    for n, pc in enumerate(capillary_pressures):
        # Multiphase.get_probe_radius (multiphase.py:98-116)
        radius = 0 if pc == 0 else 2.0 * gamma / pc * np.cos(np.deg2rad(theta))
        if method == "extended_contact_angle":
            radius = [radius, radius * np.abs(np.cos(np.deg2rad(theta)))]
            lo, hi = min(radius), max(radius)
        else:
            lo = hi = radius
        if lo < min(geom.resolution):
            morph = np.zeros_like(pm_img, dtype=np.uint8)
        else:
            if dmax is None:
                dmax = max_distance(geom, pm_img)
            if hi > dmax:
                morph = np.zeros_like(pm_img, dtype=np.uint8)
            else:
                morph = porosimetry(geom, pm_img, radius, inlet=True, mp_img=mp_img, mode=mode)
        w = outlet_connected_img(geom, mp_img, 2)
        mp_img = np.where((morph == 1) & (w == 2), 1, mp_img)
        mp_img = geom.update_reservoir(mp_img, mp_img.dtype.type(1))
        own = mp_img[geom.own_slices()]
        sat[n] = float(np.count_nonzero(own == 2) / np.prod(geom.voxels)) / phi
    return sat, mp_img


def pore_size_distribution(geom: Geom, pm_img, radii, inlet=False, mode="distance"):
    """pore_size_distribution with explicit radii (porosimetry.py:163-227)."""
    if isinstance(radii, (int, float)):
        radii = [radii]
    elif isinstance(radii, list):
        radii = sorted(radii, reverse=True)
    else:
        radii = np.sort(np.asarray(radii))[::-1]
    out = np.zeros_like(pm_img, dtype=np.double)
    for radius in radii:
        tmp = porosimetry(geom, pm_img, radius, inlet=inlet, mode=mode)
        if np.any(tmp):
            out = np.where((pm_img == 1) & (out == 0) & (tmp == 1), radius, out)
    return out


# --------------------------------------------------------------------------
# Sphere voxelisation
# --------------------------------------------------------------------------

def sphere_fill(spheres, coords):
    """gen_sphere_img_brute_force over the padded grid (before the halo update)."""
    sph = np.ascontiguousarray(spheres, dtype=np.float64).reshape(-1, 4)
    cx, cy, cz = (np.ascontiguousarray(c, dtype=np.float64) for c in coords)
    shape = np.array([cx.shape[0], cy.shape[0], cz.shape[0]], dtype=np.int64)
    img = np.empty(tuple(shape), dtype=np.uint8)
    lib().or_spheres(_ptr(sph), sph.shape[0], _ptr(cx), _ptr(cy), _ptr(cz), _ptr(img), _ptr(shape))
    return img


def gen_pm_spheres_domain(geom: Geom, spheres, invert=False):
    """gen_pm_spheres_domain, domain_generation.py:125-155 (kd=False)."""
    img = sphere_fill(spheres, geom.coords())
    img = update_buffer(geom, img)
    if invert:
        img = np.logical_not(img).astype(np.uint8)
    return geom.set_wall_bcs(img)
