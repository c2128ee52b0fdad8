"""The schedule network's CPU oracle is pinned by finite differences: its
convolution and head gradients equal central differences of its forward
functions (float64), so the GPU kernels can be checked against it."""

import numpy as np

from oracle import cnn


def test_conv_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    for d, cin, cout in [(5, 1, 3), (4, 2, 3)]:
        x = rng.standard_normal((2, d, d, d, cin))
        w = rng.standard_normal((cout, cin, 27))
        b = rng.standard_normal(cout)
        do = (d + 1) // 2
        dz = rng.standard_normal((2, do, do, do, cout))
        dx, dw, db = cnn.conv_bwd(x, w, dz)
        f = lambda x_, w_, b_: float((cnn.conv_fwd(x_, w_, b_) * dz).sum())  # noqa: E731
        h = 1e-6
        for _ in range(6):
            i = tuple(rng.integers(0, s) for s in x.shape)
            xp, xm = x.copy(), x.copy()
            xp[i] += h
            xm[i] -= h
            assert abs((f(xp, w, b) - f(xm, w, b)) / (2 * h) - dx[i]) < 1e-6 * (1 + abs(dx[i]))
            j = tuple(rng.integers(0, s) for s in w.shape)
            wp, wm = w.copy(), w.copy()
            wp[j] += h
            wm[j] -= h
            assert abs((f(x, wp, b) - f(x, wm, b)) / (2 * h) - dw[j]) < 1e-6 * (1 + abs(dw[j]))
        k = int(rng.integers(0, cout))
        bp, bm = b.copy(), b.copy()
        bp[k] += h
        bm[k] -= h
        assert abs((f(x, w, bp) - f(x, w, bm)) / (2 * h) - db[k]) < 1e-6 * (1 + abs(db[k]))


def test_head_gradients_match_finite_differences():
    rng = np.random.default_rng(1)
    y4 = np.abs(rng.standard_normal((3, 64, 64)))
    w5, b5 = rng.standard_normal((64, 64)) * 0.1, rng.standard_normal(64) * 0.1
    w6, b6 = rng.standard_normal((64, 64)) * 0.1, rng.standard_normal(64) * 0.1
    t = rng.random((3, 64))
    dy4, dw5, db5, dw6, db6 = cnn.head_bwd(y4, w5, b5, w6, b6, t)
    h = 1e-6
    for arr, grad, idx in [(w5, dw5, (3, 7)), (b5, db5, (5,)), (w6, dw6, (10, 2)), (b6, db6, (9,)),
                           (y4, dy4, (1, 4, 6))]:
        p, m = arr.copy(), arr.copy()
        p[idx] += h
        m[idx] -= h
        args = {id(w5): 1, id(b5): 2, id(w6): 3, id(b6): 4, id(y4): 0}[id(arr)]

        def L(v):
            a = [y4, w5, b5, w6, b6]
            a[args] = v
            return cnn.head_loss(*a, t)

        fd = (L(p) - L(m)) / (2 * h)
        assert abs(fd - grad[idx]) < 1e-6 * (1 + abs(grad[idx]))


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.3, 0.0], dtype=np.float32)
    r = cnn.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125  # ties to even, then up
    assert abs(r[3] + 3.3) < 0.02 and r[4] == 0.0
