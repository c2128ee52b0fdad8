"""Train the schedule network on exact curves (run on a GPU host)::

    python -m pmmoto_gb300.learned.train --samples 20000 --epochs 24 \\
        --out pmmoto_gb300/learned/weights.pt --log train_log.json

Generates the (input, curve) pairs with ``data.make_examples`` (GRF media of
the large-configuration generator with sigma, porosity and size varied, in
the drainage geometry), holds out 5 % for validation, and trains with Adam
(batch 64, cosine-decayed learning rate) on the library's kernels.  The
weights, the Adam moments and the step count are saved (``ScheduleNet.save``)
so that ``--resume`` continues a run.
"""

from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np
import torch

from . import data
from .net import ScheduleNet


def train(net, X, Y, epochs, batch=64, lr=1e-3, val_frac=0.05, seed=0, log=None):
    n = X.shape[0]
    nval = max(1, int(n * val_frac))
    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    perm = torch.randperm(n, generator=g).to(X.device)
    val, tr = perm[:nval], perm[nval:]
    steps_per_epoch = max(1, tr.numel() // batch)
    total = epochs * steps_per_epoch
    hist = []
    for ep in range(epochs):
        t0 = time.time()
        order = tr[torch.randperm(tr.numel(), generator=g).to(X.device)]
        acc = torch.zeros(1, device=X.device)
        for s in range(steps_per_epoch):
            step = ep * steps_per_epoch + s
            lr_s = lr * 0.5 * (1.0 + math.cos(math.pi * step / total))
            idx = order[s * batch:(s + 1) * batch]
            acc += net.train_step(X[idx], Y[idx], lr=lr_s)
        net.check_status()
        vl = evaluate_loss(net, X[val], Y[val], batch)
        rec = {"epoch": ep + 1, "train_loss": float(acc.item()) / steps_per_epoch, "val_loss": vl,
               "val_max_abs": val_max_abs(net, X[val], Y[val], batch), "s": round(time.time() - t0, 2)}
        hist.append(rec)
        if log:
            log(rec)
    return hist


@torch.no_grad()
def evaluate_loss(net, X, Y, batch=64):
    tot, cnt = 0.0, 0
    for i in range(0, X.shape[0], batch):
        p = net.predict(X[i:i + batch])
        tot += float(((p - Y[i:i + batch]) ** 2).mean(dim=1).sum().item())
        cnt += p.shape[0]
    return tot / max(1, cnt)


@torch.no_grad()
def val_max_abs(net, X, Y, batch=64):
    m = 0.0
    for i in range(0, X.shape[0], batch):
        p = net.predict(X[i:i + batch])
        m = max(m, float((p - Y[i:i + batch]).abs().max().item()))
    return m


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=20000)
    ap.add_argument("--epochs", type=int, default=24)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default="weights.pt")
    ap.add_argument("--resume", default=None)
    ap.add_argument("--log", default=None)
    args = ap.parse_args()
    log = {"args": vars(args), "epochs": []}

    def dump():
        if args.log:
            with open(args.log, "w") as f:
                json.dump(log, f, indent=1)

    t0 = time.time()
    X, Y, meta = data.make_examples(args.samples, seed=args.seed,
                                    log=lambda i: print(f"examples {i} {time.time() - t0:.1f}s", flush=True)
                                    if i % 1024 < 16 else None)
    torch.cuda.synchronize()
    log["data_s"] = round(time.time() - t0, 1)
    log["data_timing_s"] = {k: round(v, 2) for k, v in getattr(data.make_examples, "timing", {}).items()}
    log["data"] = {"samples": int(X.shape[0]), "r_max_vox": [float(np.min([m[4] for m in meta])),
                                                             float(np.max([m[4] for m in meta]))],
                   "mean_curve": Y.mean(0).cpu().tolist()}
    dump()
    net = ScheduleNet(seed=args.seed) if not args.resume else ScheduleNet.load(args.resume)
    t1 = time.time()

    def rec(r):
        log["epochs"].append(r)
        print(json.dumps(r), flush=True)
        dump()

    train(net, X, Y, args.epochs, batch=args.batch, lr=args.lr, seed=args.seed, log=rec)
    log["train_s"] = round(time.time() - t1, 1)
    net.save(args.out)
    dump()


if __name__ == "__main__":
    main()
