#!/usr/bin/env python
"""Benchmark of the GB300 voxel-morphology path.

Workload (one "step" = one dense exact drainage curve): a 512^3 sphere pack
(3,000 spheres, centres uniform in the unit box, radii uniform in
[0.02, 0.05]) padded to 512 x 514 x 514, walls on the y and z faces, inlet at
x = 0 and outlet at x = max; 40 probe radii uniform from 1 to 20 voxels
(capillary pressures 2 / (r * res)), each radius running erosion by the EDT,
inlet-connected components, the multiphase constraint, dilation, the
outlet-connected wetting phase and the saturation count -- PMMoTo's
drainage(..., mode="distance") with the standard method.  Inputs are
synthetic (seeded), the image stays resident in HBM for `value`; `e2e` feeds
host buffers through the package's C ABI each step.

Prints one JSON line, which also carries the large EDT + connected-components
configuration (1024^3 periodic Gaussian-random-field medium: Gvox/s and the
HBM roofline fraction of each operator).  `--impl reference` times the CPU
restatement of the same path (the oracle, all host threads) over whole
curves in sweep order.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_VOX = 512
N_SPHERES = 3000
R_LO, R_HI = 0.02, 0.05
N_RADII = 40
METRIC = "drainage curves/s (dense exact, 40 radii, 512^3 pack)"
UNIT = "curves/s"


def workload_config():
    return {"workload": "sphere-pack drainage 512^3 (512x514x514 padded), 3000 spheres r~U[0.02,0.05], "
                        "walls y/z, inlet x-, outlet x+, 40 radii linspace(1,20) voxels, mode=distance",
            "voxels": [N_VOX, N_VOX + 2, N_VOX + 2], "spheres": N_SPHERES, "radii": N_RADII,
            "l2": "inputs larger than L2 (135 MB uint8 image, 1.1 GB float32 EDT scratch per pass)"}


def make_pack(seed):
    rng = np.random.default_rng(seed)
    return np.c_[rng.random((N_SPHERES, 3)), rng.uniform(R_LO, R_HI, N_SPHERES)]


def radii_for(res):
    r_vox = np.linspace(1, 20, N_RADII)
    pcs = sorted(list(2.0 / (r_vox * res)))
    return pcs, [2.0 * 1 / pc * np.cos(np.deg2rad(0)) for pc in pcs]


def geom_kwargs():
    return dict(box=((0.0, 1.0),) * 3, boundary_types=(("end", "end"), ("wall", "wall"), ("wall", "wall")),
                inlet=((True, False), (False, False), (False, False)),
                outlet=((False, True), (False, False), (False, False)))


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def prof_read(L):
    names = ctypes.create_string_buffer(8192)
    cap = 64
    ms = (ctypes.c_double * cap)()
    by = (ctypes.c_double * cap)()
    n = (ctypes.c_longlong * cap)()
    cnt = ctypes.c_int32(0)
    L.pmg_prof_read(names, 8192, ms, by, n, cap, ctypes.byref(cnt))
    keys = names.value.decode().split("\n")
    return {keys[i]: {"ms": ms[i], "bytes": by[i], "launches": n[i]} for i in range(cnt.value)}


def max_over_ranks(x, dist, device):
    """Largest x over the ranks: the job's time is its slowest replica's."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_gpu(args):
    import torch

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import pmmoto_gb300 as P
    from pmmoto_gb300 import _lib
    from pmmoto_gb300.filters import equilibrium_distribution as ED

    L = _lib.lib()
    L.pmg_launch_count.restype = ctypes.c_longlong
    sd = P.initialize((N_VOX,) * 3, **geom_kwargs())
    sph = make_pack(1234 + rank)
    t_setup = time.time()
    pm_t = P.domain_generation.gen_pm_spheres_domain(sd, torch.as_tensor(sph, device="cuda"))
    pm = P.domain_generation.PorousMedia(sd, pm_t.img)
    mp0 = P.domain_generation.gen_mp_constant(pm, 2)
    pcs, radii = radii_for(sd.domain.resolution[0])
    _ = pm.max_distance  # cached once per medium, as PorousMedia caches it
    phi = pm.porosity
    setup_s = time.time() - t_setup

    def step():
        mp = P.domain_generation.Multiphase(pm, mp0.img, 2)
        counts, _ = ED.drainage_counts(mp, radii, mode="distance")
        return counts

    for _ in range(args.warmup):
        counts = step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = L.pmg_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        e0.record()
        for _ in range(args.steps):
            counts = step()
        e1.record()
        torch.cuda.synchronize()
    launches = L.pmg_launch_count() - n0
    ms = e0.elapsed_time(e1)
    # per-kernel CUDA events (one pair per launch, on the launching stream)
    # perturb the sweep, so they are taken over a repeat of the timed steps
    L.pmg_prof_reset()
    L.pmg_prof_enable(1)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record()
    for _ in range(args.steps):
        step()
    p1.record()
    torch.cuda.synchronize()
    L.pmg_prof_enable(0)
    prof_ms = p0.elapsed_time(p1)
    prof = prof_read(L)
    if dist:
        ms = max_over_ranks(ms, dist, "cuda")
        dist.barrier()
    sat = [float(c / np.prod(sd.domain.voxels)) / phi for c in counts]

    # end to end: host image in pinned memory -> device, drainage, saturations back
    host_pm = torch.empty(pm_t.img.shape, dtype=torch.uint8, pin_memory=True)
    host_pm.copy_(pm_t.img.cpu())
    host_mp = torch.empty_like(host_pm, pin_memory=True)
    host_mp.copy_(mp0.img.cpu())
    dev_pm = torch.empty_like(pm_t.img)
    dev_mp = torch.empty_like(pm_t.img)

    def e2e_step():
        dev_pm.copy_(host_pm, non_blocking=True)
        dev_mp.copy_(host_mp, non_blocking=True)
        # a new medium each step: its porosity and maximum distance (one EDT)
        # are computed here, as drainage needs them
        pm_e = P.domain_generation.PorousMedia(sd, dev_pm)
        mp_e = P.domain_generation.Multiphase(pm_e, dev_mp, 2)
        c, _ = ED.drainage_counts(mp_e, radii, mode="distance")
        phi_e = pm_e.porosity
        return [float(x / np.prod(sd.domain.voxels)) / phi_e for x in c]  # counts came back to the host

    e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sat_e = e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist:
        e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    assert sat_e == sat, "end-to-end path disagrees with the resident path"

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_kind = load_peaks()
    top = max(prof.items(), key=lambda kv: kv[1]["ms"]) if prof else ("none", {"ms": 1, "bytes": 0, "launches": 1})
    ach = top[1]["bytes"] / (top[1]["ms"] / 1e3) / 1e9 if top[1]["ms"] > 0 else 0.0
    traffic = load_traffic(top[0])
    total_prof_ms = sum(v["ms"] for v in prof.values())
    out = {
        "metric": METRIC, "value": world * args.steps / (ms / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(), parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
        "clocks": clk.summary(),
        "e2e": {"value": world * args.steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(host_pm.numel() * 2), "d2h_bytes_per_step": int(8 * N_RADII)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": top[0], "achieved": round(ach, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(ach / peak, 4), "peak_kind": peak_kind,
                     "traffic": traffic, "launches": int(top[1]["launches"]),
                     "avg_launch_ms": top[1]["ms"] / max(1, top[1]["launches"]),
                     "share": round(top[1]["ms"] / total_prof_ms, 3) if total_prof_ms else None,
                     "region": "profiled repeat of the timed steps",
                     "repeat_ms_per_step": prof_ms / args.steps},
        "kernels": {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                        "GBps": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1) if v["ms"] > 0 else None}
                    for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])},
        "saturation_first_last": [sat[0], sat[-1]],
        "porosity": phi,
        "setup_s": round(setup_s, 3),
    }
    if not args.no_large:
        out["edt_cc_1024"] = measure_large(args, local, peak, peak_kind)
    if not args.no_learned:
        out["learned_schedule"] = measure_learned(args)
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(sd_voxels=sd.voxels, pm_img=pm_t.img.cpu().numpy(), pcs=pcs)
    print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def load_traffic(kernel):
    p = os.path.join(REPO, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    v = d.get(kernel)
    return v.get("bytes_per_launch") if isinstance(v, dict) else None


# ---------------------------------------------------------------------------
# CPU baseline (the oracle: CPU restatement of the reference, all host threads)
# ---------------------------------------------------------------------------

SAMPLE_IDX = (0, 10, 20, 30)


def cpu_baseline(sd_voxels=None, pm_img=None, pcs=None):
    """The oracle (OpenMP C restatement of the reference) on a stratified
    sample of the curve: radii #0, #10, #20, #30 evaluated in sweep order with
    the multiphase image carried from one to the next, plus the per-medium
    porosity and maximum distance; the radii's time is scaled x10 to a
    curve."""
    from oracle import oracle as O

    L = O.lib()
    L.or_num_threads.restype = ctypes.c_int
    cores = int(L.or_num_threads())
    g = O.Geom((N_VOX,) * 3, **{k: v for k, v in geom_kwargs().items()})
    if pm_img is None:
        pm_img = O.gen_pm_spheres_domain(g, make_pack(1234))
    if pcs is None:
        pcs, _ = radii_for(g.resolution[0])
    sample = [pcs[i] for i in SAMPLE_IDX]
    t0 = time.perf_counter()
    dmax = O.max_distance(g, pm_img)  # once per medium (PorousMedia caches it)
    phi = O.porosity(g, pm_img)
    t1 = time.perf_counter()
    O.drainage(g, pm_img, sample, dmax=dmax, phi=phi)
    t2 = time.perf_counter()
    scale = N_RADII / len(sample)
    per_curve = (t1 - t0) + (t2 - t1) * scale
    return {"value": 1.0 / per_curve, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"radii #{list(SAMPLE_IDX)} of the 40 (sweep order, multiphase state carried between "
                      f"them) of the same 512^3 drainage, {t2 - t1:.1f} s scaled x{scale:g}, plus the "
                      f"medium's porosity and max distance ({t1 - t0:.1f} s, once per curve)"}


def run_reference(args):
    """Reference arm: the CPU path (the oracle port, all host threads) times
    whole curves of the same workload in sweep order with carried state.  The
    K timed steps split ceil(K / 40) curves into K runs of consecutive radii,
    each step continuing from the multiphase image the previous one left; the
    first step of every curve also computes the medium's porosity and maximum
    distance.  Nothing is extrapolated: value = curves / total time."""
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    from oracle import oracle as O

    L = O.lib()
    L.or_num_threads.restype = ctypes.c_int
    cores = int(L.or_num_threads())
    g = O.Geom((N_VOX,) * 3, **geom_kwargs())
    pm_img = O.gen_pm_spheres_domain(g, make_pack(1234))
    pcs, _ = radii_for(g.resolution[0])
    n_curves = max(1, -(-args.steps // N_RADII))
    seq = [(c, k) for c in range(n_curves) for k in range(N_RADII)]
    bounds = np.linspace(0, len(seq), args.steps + 1).round().astype(int)
    # the CPU path has nothing to warm up; one porosity count touches the image
    for _ in range(min(args.warmup, 1)):
        O.porosity(g, pm_img)
    step_s = []
    mp, dmax, phi, sat = None, None, None, []
    t_all = time.perf_counter()
    for i in range(args.steps):
        t0 = time.perf_counter()
        part = seq[bounds[i]:bounds[i + 1]]
        for c, k in part:
            if k == 0:
                mp = None
                dmax = O.max_distance(g, pm_img)
                phi = O.porosity(g, pm_img)
                sat = []
            s_k, mp = O.drainage(g, pm_img, [pcs[k]], dmax=dmax, mp_img=mp, phi=phi)
            sat.append(float(s_k[0]))
        step_s.append(time.perf_counter() - t0)
    total = time.perf_counter() - t_all
    v = n_curves / total
    cb = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
          "sample": f"{n_curves} whole 40-radius curve(s) of the 512^3 drainage in sweep order with carried "
                    f"state, split over the {args.steps} timed steps ({total:.1f} s)"}
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": dict(workload_config(), parallelism="single GPU" if world == 1 else f"replicas x{world}"),
           "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "saturation_first_last": [sat[0], sat[-1]] if sat else None,
           "step_s_min_max": [min(step_s), max(step_s)]}
    print(json.dumps(out), flush=True)


def measure_learned(args):
    """Learned radius schedule against the dense exact sweep: 12 held-out 512^3
    sphere packs of this configuration's generator (seeds the timed curve does
    not use), 64 radii r_max (k + 1) / 64; per pack the dense curve (64 exact
    radii) and the learned curve (schedule network + at most 12 exact radii,
    dense fallback on a failed residual check) are each timed from the pore
    image on the device to the curve on the host, the medium's distance
    transform included; curves/s over the packs and the largest |dS| of the
    learned curve against the dense one."""
    import os

    from pmmoto_gb300.learned import evaluate, schedule

    if not os.path.exists(schedule.default_weights_path()):
        return {"status": "no trained weights in the package"}
    sched = schedule.LearnedSchedule(schedule.load_default())
    res = evaluate.run(packs=args.learned_packs, grfs=0, seed0=7000, sched=sched)["sphere512"]["summary"]
    res["workload"] = (f"{args.learned_packs} held-out 512^3 packs (3000 spheres r~U[0.02,0.05], walls y/z, inlet x-, "
                       "outlet x+), 64 radii r_max (k+1)/64; learned <= 12 exact radii + dense fallback")
    res["target"] = {"max_abs_dS": 0.01, "speedup": 5.0}
    return res


def measure_large(args, local, peak, peak_kind):
    """Large EDT + connected-components configuration: the 1024^3 Gaussian
    random field medium (sigma 4 voxels, porosity 0.35, periodic), its
    periodic squared edt3d (own volume) and its connected components (labels
    of the padded 1026^3 periodic subdomain image, seam merge and numbering
    included), each timed over `steps` calls after `warmup` with CUDA events
    and clocks sampled; Gvox/s per voxel of the operator's input, achieved
    GB/s = algorithmic bytes (EDT 21 B, CC 17 B per voxel) / time."""
    import torch

    import pmmoto_gb300 as P
    from pmmoto_gb300 import _lib
    from pmmoto_gb300.core.geometry import geo_of
    from pmmoto_gb300.domain_generation import grf
    from pmmoto_gb300.filters import connected_components as CC
    from pmmoto_gb300.filters import distance as D

    n = 1024
    from pmmoto_gb300 import tune

    tuned = tune.tune_edt((n, n, n))  # launch parameters of this shape class (cached)
    own = grf.gen_grf_medium(n)
    idx = torch.arange(-1, n + 1, device="cuda") % n
    img = own[idx][:, idx][:, :, idx].contiguous()
    torch.cuda.synchronize()
    out = torch.empty(own.shape, dtype=torch.float32, device="cuda")
    cfg = D.edt3d_cfg((True, True, True))
    res = np.ones(3, np.float32)
    sd = P.initialize((n,) * 3, boundary_types=(("periodic", "periodic"),) * 3)
    geo = geo_of(sd)
    L = _lib.lib()
    ops = {"edt": (lambda: D.edt3d_device(own, res, cfg, True, out), own.numel(), 21.0),
           "cc": (lambda: CC.connect_components_device(img, geo), img.numel(), 17.0)}
    res_out = {"workload": "1024^3 GRF medium (sigma 4, porosity 0.35, periodic); edt3d squared on the own "
                           "1024^3 volume, connected components on the padded 1026^3 image",
               "edt_tuned": tuned,
               "l2": "inputs larger than L2 (1 GB image, 4 GB distances, 8.6 GB labels)"}
    steps = max(3, min(args.steps, 10))
    for name, (op, vox, bpv) in ops.items():
        for _ in range(max(3, args.warmup)):
            op()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = L.pmg_launch_count()
        with Clocks(local) as clk:
            e0.record()
            for _ in range(steps):
                op()
            e1.record()
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        launches = (L.pmg_launch_count() - n0) // steps
        L.pmg_prof_reset()
        L.pmg_prof_enable(1)
        op()
        torch.cuda.synchronize()
        L.pmg_prof_enable(0)
        prof = prof_read(L)
        ach = bpv * vox / (ms / 1e3) / 1e9
        res_out[name] = {"ms": round(ms, 3), "gvox_s": round(vox / ms / 1e6, 2), "voxels": vox,
                         "bytes_per_voxel": bpv, "achieved_GBps": round(ach, 1), "peak": peak,
                         "peak_kind": peak_kind, "frac": round(ach / peak, 4), "launches_per_call": launches,
                         "clocks": clk.summary(), "steps": steps,
                         "kernels": {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                                         "GBps": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1) if v["ms"] else None}
                                     for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}}
    del own, img, out
    torch.cuda.empty_cache()
    return res_out


def batch_packs(count, seed=99):
    """The batched configuration's packs: per-axis sizes drawn from {64, 96,
    ..., 256}, box N_i / 256 (voxel size 2^-8), porosity target U[0.3, 0.5],
    sphere radii U[0.02, 0.06], sphere count -ln(phi) V / (4/3 pi E[r^3]);
    returns [(voxels, spheres)]."""
    rng = np.random.default_rng(seed)
    sizes = np.arange(64, 257, 32)
    er3 = (0.06 ** 4 - 0.02 ** 4) / (4 * 0.04)
    packs = []
    for _ in range(count):
        vox = tuple(int(v) for v in rng.choice(sizes, 3))
        box = [v / 256.0 for v in vox]
        vol = box[0] * box[1] * box[2]
        phi = rng.uniform(0.3, 0.5)
        n = max(1, int(round(-np.log(phi) * vol / (4.0 / 3.0 * np.pi * er3))))
        sph = np.empty((n, 4))
        for d in range(3):
            sph[:, d] = rng.random(n) * box[d]
        sph[:, 3] = rng.uniform(0.02, 0.06, n)
        packs.append((vox, sph))
    return packs


def run_batch(args):
    """Batched configuration: EDT + connected components + 24-radius drainage
    for every pack, packs spread over CUDA streams (pmmoto_gb300.batch)."""
    import torch

    import pmmoto_gb300 as P
    from pmmoto_gb300 import _lib, batch
    from pmmoto_gb300.filters import connected_components as CC
    from pmmoto_gb300.filters import equilibrium_distribution as ED

    L = _lib.lib()
    L.pmg_launch_count.restype = ctypes.c_longlong
    packs = batch_packs(args.packs)
    media = []
    for vox, sph in packs:
        kw = geom_kwargs()
        kw["box"] = tuple((0.0, v / 256.0) for v in vox)
        sd = P.initialize(vox, **kw)
        pm = P.domain_generation.gen_pm_spheres_domain(sd, torch.as_tensor(sph, device="cuda"))
        media.append((sd, pm))
    r_vox = np.linspace(1, 12, 24)
    pcs = sorted(list(2.0 / (r_vox * 2.0 ** -8)))
    torch.cuda.synchronize()

    def one(item):
        sd, pm = item
        medium = P.domain_generation.PorousMedia(sd, pm.img)
        _ = medium.max_distance  # EDT of the pore space + halo update, as drainage needs it
        labels, nlab = CC.connect_components(pm.img, sd)
        mp = P.domain_generation.gen_mp_constant(medium, 2)
        sat = ED.drainage(mp, pcs, mode="distance")
        return float(sat[-1]), int(nlab)

    workers = args.workers
    tuned = None
    if workers <= 0:  # autotune the stream count on the first 64 packs (cached per shape class)
        from pmmoto_gb300 import tune

        items = [(p[0], m) for p, m in zip(packs, media)][:64]
        tuned = tune.tune_batch(items, lambda it: one(it[1]))
        workers = tuned["batch.workers"]
    for _ in range(args.warmup):
        batch.map_streams(one, media, workers=workers)
    torch.cuda.synchronize()
    n0 = L.pmg_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    t0 = time.time()
    for _ in range(args.steps):
        res = batch.map_streams(one, media, workers=workers)
    e1.record()
    torch.cuda.synchronize()
    wall = (time.time() - t0) / args.steps
    launches = (L.pmg_launch_count() - n0) // args.steps
    vox = sum(int(np.prod([v + 2 for v in p[0]])) for p in packs)
    print(json.dumps({"case": "batch", "packs": len(packs), "workers": workers, "tuned": tuned,
                      "metric": "batched packs/s (EDT + CC + 24-radius drainage per pack)",
                      "value": len(packs) / wall, "unit": "packs/s", "ms_per_batch": wall * 1e3,
                      "gpu_ms_per_batch": e0.elapsed_time(e1) / args.steps, "voxels": vox,
                      "gpu_launches_per_batch": launches, "final_saturation_sample": res[0][0]}), flush=True)


def run_cnn(args):
    """Schedule network on the tensor cores: one training step (forward,
    backward, Adam) on a synthetic batch of `--batch` 64^3 inputs, timed with
    CUDA events; per-kernel TFLOP/s = algorithmic flops (2 x MACs of each
    convolution; dgrad counts the 1/8 of taps that a stride-2 transpose
    touches) / CUDA-event time, against the measured dense bf16 peak."""
    import torch

    from pmmoto_gb300 import _lib
    from pmmoto_gb300.learned import ScheduleNet

    torch.manual_seed(0)
    x = torch.rand((args.batch, 64 ** 3), device="cuda").to(torch.bfloat16)
    y = torch.rand((args.batch, 64), device="cuda")
    net = ScheduleNet(seed=0)
    for _ in range(max(3, args.warmup)):
        net.train_step(x, y)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        net.train_step(x, y)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    L = _lib.lib()
    L.pmg_prof_reset()
    L.pmg_prof_enable(1)
    for _ in range(args.steps):
        net.train_step(x, y)
    torch.cuda.synchronize()
    L.pmg_prof_enable(0)
    prof = prof_read(L)
    net.check_status()
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    peak = json.load(open(p))["bf16_tflops"] if os.path.exists(p) else 1900.0
    print(json.dumps({"case": "cnn", "batch": args.batch, "ms_per_train_step": ms,
                      "samples_s": args.batch / (ms / 1e3), "bf16_peak_tflops": peak,
                      "kernels": {k: {"ms_per_step": v["ms"] / args.steps, "launches": v["launches"],
                                      "TFLOPs": v["bytes"] / (v["ms"] / 1e3) / 1e12 if v["ms"] else None,
                                      "frac": v["bytes"] / (v["ms"] / 1e3) / 1e12 / peak if v["ms"] else None}
                                  for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}}), flush=True)


def run_case(args):
    """Single-operator cases on a seeded random medium (for ncu captures and
    per-operator rates): 'edt' = edt3d, 'cc' = connected components (with the
    periodic merge when --bc periodic), 'morph' = erosion (EDT path); N^3
    voxels, all faces periodic or all walls (--bc); 'select' = inlet-connected
    pore space of the drainage pack (its geometry, N-2 own voxels per axis)."""
    import torch

    import pmmoto_gb300 as P
    from pmmoto_gb300 import _lib
    from pmmoto_gb300.filters import connected_components as CC
    from pmmoto_gb300.filters import distance as D
    from pmmoto_gb300.filters import morphological_operators as M
    from pmmoto_gb300.core.geometry import geo_of

    n = args.n
    if args.medium == "grf":
        from pmmoto_gb300.domain_generation import grf

        img = grf.gen_grf_medium(n)
    else:
        g = torch.Generator(device="cuda")
        g.manual_seed(7)
        img = (torch.rand((n, n, n), device="cuda", generator=g) >= 0.35).to(torch.uint8)
    per = args.bc == "periodic"
    # voxel size 1/512 (a power of two, like the drainage pack)
    sd = P.initialize((n - 2,) * 3, box=((0.0, (n - 2) / 512.0),) * 3, boundary_types=((args.bc, args.bc),) * 3)
    geo = geo_of(sd)
    out = torch.empty((n, n, n), dtype=torch.float32, device="cuda")
    cfg = D.edt3d_cfg((per, per, per))
    res = np.ones(3, np.float32)

    if args.case == "select":
        # inlet-connected pore space of the drainage pack geometry (walls y/z,
        # inlet x-), binary 2x2x2-block labelling
        kw = geom_kwargs()
        kw["box"] = ((0.0, (n - 2) / 512.0),) * 3
        sd = P.initialize((n - 2,) * 3, **kw)
        geo = geo_of(sd)
        pm = P.domain_generation.gen_pm_spheres_domain(sd, torch.as_tensor(make_pack(1234), device="cuda"))
        img = pm.img

    def op():
        if args.case == "select":
            CC.select_device(geo, img, CC.SEL_INLET | CC.SEL_BINARY)
        elif args.case == "edt":
            D.edt3d_device(img, res, cfg, True, out)
        elif args.case == "cc":
            CC.connect_components_device(img, geo)
        else:
            M.morph_device(geo, img, 4.0 * sd.domain.resolution[0], False)

    for _ in range(args.warmup):
        op()
    torch.cuda.synchronize()
    L = _lib.lib()
    L.pmg_prof_reset()
    L.pmg_prof_enable(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        op()
    e1.record()
    torch.cuda.synchronize()
    L.pmg_prof_enable(0)
    ms = e0.elapsed_time(e1) / args.steps
    prof = prof_read(L)
    peak, _ = load_peaks()
    print(json.dumps({"case": args.case, "bc": args.bc, "medium": args.medium, "n": n, "ms": ms, "gvox_s": n**3 / ms / 1e6,
                      "kernels": {k: {"ms_per_step": v["ms"] / args.steps, "launches": v["launches"],
                                      "GBps": v["bytes"] / (v["ms"] / 1e3) / 1e9 if v["ms"] else None,
                                      "frac": v["bytes"] / (v["ms"] / 1e3) / 1e9 / peak if v["ms"] else None}
                                  for k, v in prof.items()}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--no-large", action="store_true", help="skip the 1024^3 EDT + CC measurement")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-schedule measurement")
    ap.add_argument("--learned-packs", type=int, default=12, help="held-out packs of the learned-schedule leg")
    ap.add_argument("--case", default="drainage",
                    choices=["drainage", "edt", "cc", "morph", "select", "batch", "cnn"])
    ap.add_argument("--batch", type=int, default=64, help="samples per training step of the cnn case")
    ap.add_argument("--packs", type=int, default=256, help="packs of the batched case")
    ap.add_argument("--workers", type=int, default=8,
                    help="host threads / CUDA streams of the batched case (0: autotune, cached per shape class)")
    ap.add_argument("--n", type=int, default=512, help="volume side of the single-operator cases")
    ap.add_argument("--bc", default="periodic", choices=["periodic", "wall"],
                    help="boundary type of every face in the single-operator cases")
    ap.add_argument("--medium", default="random", choices=["random", "grf"],
                    help="single-operator cases: uniform random (65%% pore) or the Gaussian random field "
                         "(sigma 4 voxels, porosity 0.35) of the large EDT + CC configuration")
    args = ap.parse_args()
    if args.case == "batch":
        run_batch(args)
    elif args.case == "cnn":
        run_cnn(args)
    elif args.case != "drainage":
        run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
