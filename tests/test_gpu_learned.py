"""The trained schedule network in the package (weights.pt, trained by
pmmoto_gb300.learned.train on 20,000 exact curves of GRF media) on media it
has not seen:

* ablation of the network: its predicted curve is much closer to the exact
  dense curve than the training set's mean curve (what the same pipeline
  has without a network) on held-out GRF media;
* the learned schedule evaluates at most 12 radii exactly (no fallback on
  these media) and returns a full, monotone 64-point curve in [0, 1];
* the dense curve it is compared with is the exact sweep, checked
  bit for bit elsewhere (test_gpu_large.py, test_gpu_workflows.py).
"""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sched():
    from pmmoto_gb300.learned import schedule

    if not os.path.exists(schedule.default_weights_path()):
        pytest.skip("no trained weights in the package")
    return schedule, schedule.LearnedSchedule(schedule.load_default())


def test_network_beats_the_mean_curve_on_held_out_media():
    from pmmoto_gb300.learned import data, evaluate

    schedule, sched = _sched()
    meta = os.path.join(os.path.dirname(schedule.default_weights_path()), "weights_meta.json")
    mean_curve = schedule.monotone(np.array(json.load(open(meta))["data"]["mean_curve"]))
    err_net, err_mean = [], []
    for seed in range(6000, 6006):
        sd, img = evaluate.grf_medium(seed)
        pm = evaluate._fresh(sd, img)
        dense = data.dense_curve(sd, pm)
        pred = schedule.monotone(sched.predict(sd, pm))
        err_net.append(np.abs(pred - dense).max())
        err_mean.append(np.abs(mean_curve - dense).max())
    assert np.mean(err_net) < 0.7 * np.mean(err_mean), (err_net, err_mean)


def test_schedule_on_a_held_out_pack():
    from pmmoto_gb300.learned import evaluate

    _, sched = _sched()
    sd, img = evaluate.sphere_pack(6100)
    pm = evaluate._fresh(sd, img)
    curve, info = sched.curve(sd, pm)
    assert curve.shape == (64,)
    assert np.all((curve >= 0) & (curve <= 1))
    assert np.all(np.diff(curve) >= -1e-12)  # saturation does not rise with the radius
    if not info["fallback"]:
        assert info["evaluations"] <= 12
        for k, v in info["exact"].items():
            assert curve[k] == v
