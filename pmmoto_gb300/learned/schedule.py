"""Learned radius schedule for the drainage curve.

The dense method evaluates all 64 radii r_k = r_max (k + 1) / 64 of the curve
(``data.radii_grid``) exactly, largest first (equilibrium_distribution.py:
93-128 sweeps every capillary pressure).  The learned method:

1. predicts the curve S^[k] with the schedule network from the medium's
   downsampled distance field (the field the max distance comes from, so it
   costs one 64^3 average and the network) and makes it non-decreasing in
   the radius;
2. plans at most ``budget`` radii: radii below the voxel size change nothing
   (the reference's skip rule), so the smallest active radius is always
   planned; the others are placed, by a greedy jump along the sweep inside a
   bisection on the largest allowed predicted drop, so that every gap that
   skips radii spans a predicted drop of at most that bound (adjacent radii
   skip nothing and may span any drop, so a predicted breakthrough jump gets
   bracketed);
3. evaluates the planned radii exactly in one native sweep (largest first,
   the multiphase image carried), i.e. the reference's loop over those
   capillary pressures;
4. fills each skipped radius from its gap's exact end values, shaped by the
   prediction: S_j = S_b + (S_a - S_b) (S^_j - S^_b) / (S^_a - S^_b);
5. residual check: when a gap that skips radii turns out to span an exact
   drop above ``fallback_drop``, the prediction misjudged that part of the
   curve, and the dense sweep is run instead (its result is returned).

``uniform_curve`` is the same pipeline without the network (planned radii
equally spaced over the active range, linear fill): the ablation.
"""

from __future__ import annotations

import numpy as np

from . import data

N_RADII = data.N_RADII


def monotone(pred: np.ndarray) -> np.ndarray:
    """Non-decreasing in the radius (running maximum from the smallest radius)."""
    return np.maximum.accumulate(np.clip(np.asarray(pred, dtype=np.float64), 0.0, 1.0))


def active_from(r_max: float, res: float) -> int:
    """Smallest grid index whose radius is not below the voxel size."""
    grid = data.radii_grid(r_max)
    idx = np.nonzero(grid >= res)[0]
    return int(idx[0]) if idx.size else N_RADII - 1


def _greedy(pred_ext, k_min, theta):
    """Planned indices (descending) with every skipping gap's predicted drop
    <= theta; pred_ext[N_RADII] = 1 is the start of the sweep."""
    plan = []
    a = N_RADII
    while a > k_min:
        b = a - 1
        # jump as far down as the bound allows (never past k_min)
        while b - 1 >= k_min and pred_ext[a] - pred_ext[b - 1] <= theta:
            b -= 1
        plan.append(b)
        a = b
    if not plan or plan[-1] != k_min:
        plan.append(k_min)
    return plan


def plan_radii(pred: np.ndarray, k_min: int, budget: int = 12):
    """At most `budget` planned indices (descending) minimising the largest
    predicted drop over gaps that skip radii."""
    p = monotone(pred)
    pred_ext = np.append(p, 1.0)
    lo, hi = 0.0, 1.0
    best = _greedy(pred_ext, k_min, hi)
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        cand = _greedy(pred_ext, k_min, mid)
        if len(cand) <= budget:
            best, hi = cand, mid
        else:
            lo = mid
    return best


def fill(exact: dict, pred: np.ndarray, k_min: int) -> np.ndarray:
    """Full 64-point curve from the exact values at the planned indices and the
    predicted shape between them (linear where the prediction is flat)."""
    p = np.append(monotone(pred), 1.0)
    known = dict(exact)
    known[N_RADII] = 1.0
    keys = sorted(known, reverse=True)
    out = np.empty(N_RADII)
    for a, b in zip(keys[:-1], keys[1:]):
        sa, sb = known[a], known[b]
        for j in range(b, min(a, N_RADII)):
            if j == b:
                out[j] = sb
            elif p[a] - p[b] > 1e-9:
                out[j] = sb + (sa - sb) * (p[j] - p[b]) / (p[a] - p[b])
            else:
                out[j] = sb + (sa - sb) * (j - b) / (a - b)
    out[:k_min] = known[k_min]
    return out


def max_skipped_drop(exact: dict, k_min: int) -> float:
    known = dict(exact)
    known[N_RADII] = 1.0
    keys = sorted(known, reverse=True)
    d = 0.0
    for a, b in zip(keys[:-1], keys[1:]):
        if a - b > 1:
            d = max(d, known[a] - known[b])
    return d


class LearnedSchedule:
    """Applies a trained ScheduleNet to media (see the module docstring)."""

    def __init__(self, net, budget: int = 12, fallback_drop: float = 0.25):
        self.net = net
        self.budget = budget
        self.fallback_drop = fallback_drop

    def predict(self, sd, pm) -> np.ndarray:
        x = data.features(sd, pm).reshape(1, -1)
        return self.net.predict(x)[0].double().cpu().numpy()

    def predicted_curve(self, sd, pm) -> np.ndarray:
        """The network's curve alone (no exact radius): monotone prediction,
        radii below the voxel size holding the smallest active radius's value."""
        k_min = active_from(float(pm.max_distance), min(sd.domain.resolution))
        c = monotone(self.predict(sd, pm))
        c[:k_min] = c[k_min]
        return c

    def curve(self, sd, pm):
        """(curve [64], info): info has the planned indices, the exact values,
        whether the dense fallback ran, and the number of exact radii."""
        r_max = float(pm.max_distance)
        k_min = active_from(r_max, min(sd.domain.resolution))
        pred = self.predict(sd, pm)
        plan = plan_radii(pred, k_min, self.budget)
        exact = data.curve_at(sd, pm, plan, r_max)
        info = {"plan": plan, "exact": exact, "k_min": k_min, "pred": pred, "evaluations": len(plan)}
        drop = max_skipped_drop(exact, k_min)
        info["max_skipped_drop"] = drop
        if drop > self.fallback_drop:
            info["fallback"] = True
            info["evaluations"] += N_RADII - k_min
            return data.dense_curve(sd, pm), info
        info["fallback"] = False
        return fill(exact, pred, k_min), info


def uniform_curve(sd, pm, budget: int = 12):
    """Ablation without the network: `budget` radii spread evenly over the
    active range (largest and smallest active radius included), linear fill."""
    r_max = float(pm.max_distance)
    k_min = active_from(r_max, min(sd.domain.resolution))
    plan = sorted(set(np.linspace(N_RADII - 1, k_min, budget).round().astype(int).tolist()), reverse=True)
    exact = data.curve_at(sd, pm, plan, r_max)
    flat = np.zeros(N_RADII)  # a flat prediction makes fill() linear
    return fill(exact, flat, k_min), {"plan": plan, "exact": exact, "evaluations": len(plan)}


def default_weights_path():
    import os

    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights.pt")


def load_default(device="cuda"):
    from .net import ScheduleNet

    return ScheduleNet.load(default_weights_path(), device=device)
