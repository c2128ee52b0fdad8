"""Host logic of the learned radius schedule (no GPU): the plan respects the
evaluation budget and always ends at the smallest active radius, a gap that
skips radii spans at most the plan's predicted-drop bound, a predicted jump
is bracketed by adjacent radii, and the fill reproduces a curve exactly when
the prediction has the curve's shape."""

import numpy as np
import pytest

from pmmoto_gb300.learned import schedule as S


def _sigmoid_curve(c, w):
    k = np.arange(64)
    return 1.0 / (1.0 + np.exp(-(k - c) / w)) * 0.7 + 0.3


@pytest.mark.parametrize("c,w,kmin", [(30, 3.0, 3), (10, 1.0, 0), (50, 0.3, 5), (40, 8.0, 2)])
def test_plan_budget_and_bounds(c, w, kmin):
    pred = _sigmoid_curve(c, w)
    plan = S.plan_radii(pred, kmin, 12)
    assert len(plan) <= 12
    assert plan == sorted(plan, reverse=True)
    assert plan[-1] == kmin
    p = np.append(S.monotone(pred), 1.0)
    keys = [64] + plan
    worst = max((p[a] - p[b]) for a, b in zip(keys[:-1], keys[1:]) if a - b > 1)
    # the uniform plan's worst predicted drop is never better than the plan's
    uni = sorted(set(np.linspace(63, kmin, 12).round().astype(int).tolist()), reverse=True)
    ukeys = [64] + uni
    uworst = max((p[a] - p[b]) for a, b in zip(ukeys[:-1], ukeys[1:]) if a - b > 1)
    assert worst <= uworst + 1e-12


def test_sharp_jump_is_bracketed():
    pred = np.where(np.arange(64) >= 37, 1.0, 0.4)
    plan = S.plan_radii(pred, 2, 12)
    assert 36 in plan and 37 in plan


def test_fill_is_exact_when_the_shape_is_right():
    true = S.monotone(_sigmoid_curve(25, 4.0))
    plan = S.plan_radii(true, 4, 12)
    exact = {k: float(true[k]) for k in plan}
    out = S.fill(exact, true, 4)
    assert np.allclose(out[4:], true[4:], atol=1e-12)
    assert np.all(out[:4] == true[4])


def test_fill_with_flat_prediction_is_linear():
    exact = {63: 0.9, 30: 0.6, 0: 0.2}
    out = S.fill(exact, np.zeros(64), 0)
    assert out[63] == 0.9 and out[30] == 0.6 and out[0] == 0.2
    assert abs(out[15] - (0.2 + 0.4 * 15 / 30)) < 1e-12
    assert S.max_skipped_drop(exact, 0) == pytest.approx(0.4)
