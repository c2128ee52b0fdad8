"""Held-out evaluation of the learned schedule (run on a GPU host)::

    python -m pmmoto_gb300.learned.evaluate --packs 50 --out eval.json

For each held-out medium, four curves over the same 64 radii:

* dense   -- all 64 radii evaluated exactly (the curve errors are measured against it);
* learned -- ``LearnedSchedule`` (at most 12 exact radii, dense fallback);
* uniform -- 12 evenly spaced exact radii, linear fill (no network);
* predicted -- the network's curve alone, no exact radius.

Media: 512^3 sphere packs of the plain-drainage configuration (3,000
spheres, radii U[0.02, 0.05], walls y/z, inlet x-, outlet x+) with seeds the
benchmark does not use, and 128^3 GRF media of the large-configuration
generator (sigma 4, porosity 0.35) in the same geometry.  Each method is
timed separately per medium (CUDA-synchronised wall clock) from the pore
image on the device to the curve on the host, including the medium's
distance transform, porosity and max distance that each method needs.
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import data, schedule


def sphere_pack(seed, n=512, count=3000, r_lo=0.02, r_hi=0.05):
    import pmmoto_gb300 as P

    rng = np.random.default_rng(seed)
    sph = np.c_[rng.random((count, 3)), rng.uniform(r_lo, r_hi, count)]
    sd = P.initialize((n,) * 3, box=((0.0, 1.0),) * 3, **data.drainage_kwargs())
    pm = P.domain_generation.gen_pm_spheres_domain(sd, torch.as_tensor(sph, device="cuda"))
    return sd, pm.img


def grf_medium(seed, n=128, sigma=4.0, porosity=0.35):
    import pmmoto_gb300 as P
    from ..domain_generation import grf

    own = grf.gen_grf_medium((n,) * 3, porosity=porosity, seed=seed, sigma=sigma)
    sd = P.initialize((n,) * 3, box=((0.0, 1.0),) * 3, **data.drainage_kwargs())
    return sd, data.padded_medium(own)


def _fresh(sd, img):
    import pmmoto_gb300 as P

    return P.domain_generation.PorousMedia(sd, img)


def _timed(fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def evaluate_medium(sd, img, sched):
    def dense():
        pm = _fresh(sd, img)
        return data.dense_curve(sd, pm)

    def learned():
        pm = _fresh(sd, img)
        return sched.curve(sd, pm)

    def uniform():
        pm = _fresh(sd, img)
        return schedule.uniform_curve(sd, pm, sched.budget)

    def predicted():
        pm = _fresh(sd, img)
        return sched.predicted_curve(sd, pm)

    sd_curve, t_dense = _timed(dense)
    pcurve, t_pred = _timed(predicted)
    (lc, linfo), t_learned = _timed(learned)
    (uc, uinfo), t_uniform = _timed(uniform)
    # the same pipeline with a perfect prediction (the dense curve itself):
    # the error left is what evaluating a subset of radii costs by itself
    pm = _fresh(sd, img)
    k_min = schedule.active_from(float(pm.max_distance), min(sd.domain.resolution))
    plan = schedule.plan_radii(sd_curve, k_min, sched.budget)
    pc = schedule.fill(data.curve_at(sd, pm, plan, float(pm.max_distance)), sd_curve, k_min)
    return {"dense_s": t_dense, "learned_s": t_learned, "uniform_s": t_uniform, "predict_s": t_pred,
            "predict_only_max_abs": float(np.abs(pcurve - sd_curve).max()),
            "perfect_plan_max_abs": float(np.abs(pc - sd_curve).max()),
            "learned_max_abs": float(np.abs(lc - sd_curve).max()),
            "uniform_max_abs": float(np.abs(uc - sd_curve).max()),
            "learned_evaluations": int(linfo["evaluations"]), "fallback": bool(linfo["fallback"]),
            "max_skipped_drop": float(linfo["max_skipped_drop"]),
            "exact_vs_dense_at_plan": float(max(abs(v - sd_curve[k]) for k, v in linfo["exact"].items())),
            "pred_max_abs": float(np.abs(schedule.monotone(linfo["pred"]) - sd_curve).max()),
            "dense": sd_curve.tolist(), "learned": lc.tolist(), "plan": [int(k) for k in linfo["plan"]]}


def summarise(rows):
    if not rows:
        return {}
    td = sum(r["dense_s"] for r in rows)
    tl = sum(r["learned_s"] for r in rows)
    tu = sum(r["uniform_s"] for r in rows)
    la = np.array([r["learned_max_abs"] for r in rows])
    ua = np.array([r["uniform_max_abs"] for r in rows])
    return {"media": len(rows), "dense_curves_s": len(rows) / td, "learned_curves_s": len(rows) / tl,
            "uniform_curves_s": len(rows) / tu, "speedup_learned_vs_dense": td / tl,
            "learned_max_abs_dS": float(la.max()), "learned_mean_max_abs_dS": float(la.mean()),
            "learned_within_0.01": int((la <= 0.01).sum()), "uniform_max_abs_dS": float(ua.max()),
            "uniform_mean_max_abs_dS": float(ua.mean()), "uniform_within_0.01": int((ua <= 0.01).sum()),
            "fallbacks": int(sum(r["fallback"] for r in rows)),
            "mean_evaluations": float(np.mean([r["learned_evaluations"] for r in rows])),
            "exact_vs_dense_at_plan_max": float(max(r["exact_vs_dense_at_plan"] for r in rows)),
            "perfect_plan_max_abs_dS": float(max(r["perfect_plan_max_abs"] for r in rows)),
            "perfect_plan_mean_max_abs_dS": float(np.mean([r["perfect_plan_max_abs"] for r in rows])),
            "pred_max_abs_mean": float(np.mean([r["pred_max_abs"] for r in rows])),
            "predict_only_curves_s": len(rows) / sum(r["predict_s"] for r in rows),
            "predict_only_max_abs_dS": float(max(r["predict_only_max_abs"] for r in rows)),
            "predict_only_mean_max_abs_dS": float(np.mean([r["predict_only_max_abs"] for r in rows]))}


def run(packs=50, grfs=50, seed0=5000, sched=None, warm=True, keep_curves=False):
    sched = sched or schedule.LearnedSchedule(schedule.load_default())
    if warm:  # first-call costs (library load, kernel attributes) outside the timings
        sd, img = grf_medium(seed0 - 1)
        evaluate_medium(sd, img, sched)
    out = {}
    for name, count, make in (("sphere512", packs, sphere_pack), ("grf128", grfs, grf_medium)):
        rows = []
        for i in range(count):
            sd, img = make(seed0 + i)
            r = evaluate_medium(sd, img, sched)
            if not keep_curves:
                for k in ("dense", "learned"):
                    r.pop(k)
            rows.append(r)
        out[name] = {"summary": summarise(rows), "media": rows}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--packs", type=int, default=50)
    ap.add_argument("--grfs", type=int, default=50)
    ap.add_argument("--weights", default=None)
    ap.add_argument("--fallback-drop", type=float, default=0.25)
    ap.add_argument("--out", default=None)
    ap.add_argument("--keep-curves", action="store_true")
    args = ap.parse_args()
    from .net import ScheduleNet

    net = ScheduleNet.load(args.weights) if args.weights else schedule.load_default()
    res = run(args.packs, args.grfs, sched=schedule.LearnedSchedule(net, fallback_drop=args.fallback_drop),
              keep_curves=args.keep_curves)
    print(json.dumps({k: v["summary"] for k, v in res.items()}, indent=1), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(res, f)


if __name__ == "__main__":
    main()
