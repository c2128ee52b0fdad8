"""Schedule-network kernels (bf16 tcgen05 convolutions, fp32 head and Adam)
against the float64 CPU oracle (oracle/cnn.py, itself pinned by finite
differences).  Operands are rounded to bf16 on both sides, so the remaining
difference is the fp32 accumulation order and the bf16 rounding of the
kernels' bf16 outputs: tolerance 1/128 of the value plus 1e-3 of the largest
magnitude for bf16 outputs, 1e-3 relative to the largest magnitude for fp32
weight gradients, 1e-4 for the fp32 head."""

import ctypes

import numpy as np
import pytest

from oracle import cnn

pytestmark = pytest.mark.gpu


def _net_lib():
    from pmmoto_gb300.learned import net

    return net.L(), net


def _t(a, dtype):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _close_bf16(got, want):
    got = np.asarray(got, np.float64)
    scale = max(1e-6, float(np.abs(want).max()))
    err = np.abs(got - want) - (np.abs(want) / 128 + 1e-3 * scale)
    assert err.max() <= 0, f"max excess {err.max():.3g} (scale {scale:.3g})"


SHAPES = [(16, 1, 16), (16, 16, 32), (8, 32, 64), (8, 64, 64), (6, 16, 16), (7, 32, 64), (64, 1, 16)]


def _packed(L, net, w, cin, cout):
    import torch

    wk = torch.zeros(cout * net._kpad(27 * cin), dtype=torch.bfloat16, device="cuda")
    wkt = torch.zeros(cin * net._kpad(27 * cout), dtype=torch.bfloat16, device="cuda") if cin >= 16 else None
    wt = _t(w, torch.float32)
    assert L.pmg_cnn_pack_weights(_p(wt), cin, cout, _p(wk), _p(wkt), _stream()) == 0
    return wk, wkt


@pytest.mark.parametrize("d,cin,cout", SHAPES)
def test_conv_forward_matches_oracle(d, cin, cout):
    import torch

    L, net = _net_lib()
    rng = np.random.default_rng(d * 100 + cin + cout)
    b = 2 if d < 64 else 1
    x = cnn.bf16(rng.standard_normal((b, d, d, d, cin)))
    w = cnn.bf16(rng.standard_normal((cout, cin, 27)) / np.sqrt(27 * cin))
    bias = rng.standard_normal(cout) * 0.1
    wk, _ = _packed(L, net, w, cin, cout)
    do = (d + 1) // 2
    y = torch.empty(b * do ** 3 * cout, dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.pmg_cnn_conv_fwd(_p(_t(x, torch.bfloat16)), _p(wk), _p(_t(bias, torch.float32)), _p(y), b, d, cin,
                              cout, _p(err), _stream()) == 0
    assert L.pmg_cnn_check(_p(err), _stream()) == 0
    want = np.maximum(cnn.conv_fwd(x, w, bias), 0.0)
    _close_bf16(y.float().cpu().numpy().reshape(want.shape), want)


@pytest.mark.parametrize("d,cin,cout", [s for s in SHAPES if s[1] >= 16])
def test_conv_dgrad_matches_oracle(d, cin, cout):
    import torch

    L, net = _net_lib()
    rng = np.random.default_rng(d * 7 + cin + cout)
    b = 2
    do = (d + 1) // 2
    w = cnn.bf16(rng.standard_normal((cout, cin, 27)) / np.sqrt(27 * cin))
    dz = cnn.bf16(rng.standard_normal((b, do, do, do, cout)))
    xact = cnn.bf16(np.maximum(rng.standard_normal((b, d, d, d, cin)), 0.0))
    _, wkt = _packed(L, net, w, cin, cout)
    dx = torch.empty(b * d ** 3 * cin, dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.pmg_cnn_conv_dgrad(_p(_t(dz, torch.bfloat16)), _p(wkt), _p(_t(xact, torch.bfloat16)), _p(dx), b, d,
                                cin, cout, _p(err), _stream()) == 0
    assert L.pmg_cnn_check(_p(err), _stream()) == 0
    want = cnn.conv_bwd(np.zeros((b, d, d, d, cin)), w, dz)[0] * (xact > 0)
    _close_bf16(dx.float().cpu().numpy().reshape(want.shape), want)


@pytest.mark.parametrize("d,cin,cout", SHAPES)
def test_conv_wgrad_matches_oracle(d, cin, cout):
    import torch

    L, net = _net_lib()
    rng = np.random.default_rng(d * 13 + cin + cout)
    b = 2 if d < 64 else 1
    do = (d + 1) // 2
    x = cnn.bf16(rng.standard_normal((b, d, d, d, cin)))
    dz = cnn.bf16(rng.standard_normal((b, do, do, do, cout)))
    dwbuf = torch.empty(27 * cin * cout, dtype=torch.float32, device="cuda")
    grad = torch.empty(cout * cin * 27, dtype=torch.float32, device="cuda")
    db = torch.empty(cout, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.pmg_cnn_conv_wgrad(_p(_t(x, torch.bfloat16)), _p(_t(dz, torch.bfloat16)), _p(dwbuf), _p(grad), _p(db),
                                b, d, cin, cout, _p(err), _stream()) == 0
    assert L.pmg_cnn_check(_p(err), _stream()) == 0
    _, dw, dbw = cnn.conv_bwd(x, np.zeros((cout, cin, 27)), dz)
    got = grad.cpu().numpy().reshape(dw.shape)
    assert np.abs(got - dw).max() <= 1e-3 * np.abs(dw).max()
    assert np.abs(db.cpu().numpy() - dbw).max() <= 1e-3 * max(1.0, np.abs(dbw).max())


def test_head_matches_oracle():
    import torch

    L, net = _net_lib()
    rng = np.random.default_rng(5)
    b = 5
    y4 = cnn.bf16(np.maximum(rng.standard_normal((b, 64, 64)), 0.0))
    w5, b5 = rng.standard_normal((64, 64)) * 0.1, rng.standard_normal(64) * 0.1
    w6, b6 = rng.standard_normal((64, 64)) * 0.1, rng.standard_normal(64) * 0.1
    t = rng.random((b, 64))
    params = _t(np.concatenate([w5.ravel(), b5, w6.ravel(), b6]), torch.float32)
    grads = torch.zeros_like(params)
    pred = torch.empty(b * 64, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    dy4 = torch.empty(b * 64 * 64, dtype=torch.bfloat16, device="cuda")
    assert L.pmg_cnn_head(_p(_t(y4, torch.bfloat16)), _p(params), b, _p(_t(t, torch.float32)), _p(pred), _p(loss),
                          _p(grads), _p(dy4), _stream()) == 0
    _, _, s = cnn.head_fwd(y4, w5, b5, w6, b6)
    assert np.abs(pred.cpu().numpy().reshape(b, 64) - s).max() < 1e-4
    assert abs(loss.item() - cnn.head_loss(y4, w5, b5, w6, b6, t)) < 1e-5
    dy, dw5, db5, dw6, db6 = cnn.head_bwd(y4, w5, b5, w6, b6, t)
    g = grads.cpu().numpy()
    want = np.concatenate([dw5.ravel(), db5, dw6.ravel(), db6])
    assert np.abs(g - want).max() < 1e-4 * max(1e-3, np.abs(want).max()) + 1e-7
    _close_bf16(dy4.float().cpu().numpy().reshape(b, 64, 64), dy * (y4 > 0))


def test_training_lowers_the_loss_and_resumes(tmp_path):
    import torch

    from pmmoto_gb300.learned import ScheduleNet

    torch.manual_seed(0)
    x = torch.rand((4, 64, 64, 64), device="cuda").to(torch.bfloat16)
    r = torch.linspace(0, 1, 64, device="cuda")
    target = torch.stack([torch.sigmoid((r - c) * 12) for c in (0.2, 0.4, 0.6, 0.8)]).contiguous()
    net = ScheduleNet(seed=1)
    first = float(net.train_step(x, target, lr=3e-3).item())
    for _ in range(40):
        last = float(net.train_step(x, target, lr=3e-3).item())
    net.check_status()
    assert last < 0.5 * first, (first, last)
    p = tmp_path / "net.pt"
    net.save(p)
    net2 = ScheduleNet.load(p)
    assert net2.step == net.step
    assert torch.equal(net2.predict(x), net.predict(x))
    # the split-K weight gradients add fp32 partial sums with atomics, whose
    # order varies between runs: equal up to that rounding
    l1 = float(net.train_step(x, target, lr=3e-3).item())
    l2 = float(net2.train_step(x, target, lr=3e-3).item())
    assert abs(l1 - l2) <= 1e-5 * abs(l1)
