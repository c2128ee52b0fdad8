"""ORACLE for the schedule network -- test infrastructure only.

Float64 numpy restatement of the network's operations (the network has no
counterpart in the reference): 3x3x3 convolution with stride 2 and padding 1
on channels-last volumes, its input and weight gradients, and the head
(global average pool, MLP 64 -> 64 -> 64 with ReLU, sigmoid, mean squared
error).  The gradients are checked against finite differences of the
forward functions on the CPU (tests/test_cnn_oracle.py); the GPU kernels are
checked against these functions.
"""

from __future__ import annotations

import numpy as np

TAPS = [(t // 9, (t // 3) % 3, t % 3) for t in range(27)]


def _windows(xp, do):
    """For each tap, the strided view of the padded input that the tap reads."""
    for t, (kz, ky, kx) in enumerate(TAPS):
        yield t, xp[:, kz:kz + 2 * do:2, ky:ky + 2 * do:2, kx:kx + 2 * do:2, :]


def conv_fwd(x, w, b):
    """x [B, D, D, D, cin], w [cout, cin, 27], b [cout] -> pre-activation
    [B, Do, Do, Do, cout], Do = (D + 1) // 2."""
    x = np.asarray(x, dtype=np.float64)
    bsz, d = x.shape[0], x.shape[1]
    do = (d + 1) // 2
    xp = np.pad(x, ((0, 0), (1, 2 * do - d), (1, 2 * do - d), (1, 2 * do - d), (0, 0)))
    z = np.zeros((bsz, do, do, do, w.shape[0]))
    for t, xs in _windows(xp, do):
        z += xs @ np.asarray(w, np.float64)[:, :, t].T
    return z + np.asarray(b, np.float64)


def conv_bwd(x, w, dz):
    """Gradients of sum(conv_fwd(x, w, b) * dz): (dx, dw, db)."""
    x = np.asarray(x, dtype=np.float64)
    d = x.shape[1]
    do = dz.shape[1]
    xp = np.pad(x, ((0, 0), (1, 2 * do - d), (1, 2 * do - d), (1, 2 * do - d), (0, 0)))
    dxp = np.zeros_like(xp)
    dw = np.zeros(w.shape)
    for t, (kz, ky, kx) in enumerate(TAPS):
        xs = xp[:, kz:kz + 2 * do:2, ky:ky + 2 * do:2, kx:kx + 2 * do:2, :]
        dw[:, :, t] = np.einsum("bzyxo,bzyxc->oc", dz, xs)
        dxp[:, kz:kz + 2 * do:2, ky:ky + 2 * do:2, kx:kx + 2 * do:2, :] += dz @ np.asarray(w, np.float64)[:, :, t]
    dx = dxp[:, 1:1 + d, 1:1 + d, 1:1 + d, :]
    db = dz.sum(axis=(0, 1, 2, 3))
    return dx, dw, db


def head_fwd(y4, w5, b5, w6, b6):
    """y4 [B, 64 positions, 64 channels] -> (pool, hidden, sigmoid output)."""
    h0 = np.asarray(y4, np.float64).mean(axis=1)
    h1 = np.maximum(h0 @ w5.T + b5, 0.0)
    s = 1.0 / (1.0 + np.exp(-(h1 @ w6.T + b6)))
    return h0, h1, s


def head_loss(y4, w5, b5, w6, b6, target):
    _, _, s = head_fwd(y4, w5, b5, w6, b6)
    return float(((s - target) ** 2).mean(axis=1).mean())


def head_bwd(y4, w5, b5, w6, b6, target):
    """Gradients of head_loss: (dy4 before the last ReLU mask, dw5, db5, dw6, db6)."""
    bsz = y4.shape[0]
    h0, h1, s = head_fwd(y4, w5, b5, w6, b6)
    dout = 2.0 * (s - target) / (s.shape[1] * bsz) * s * (1.0 - s)
    dw6, db6 = dout.T @ h1, dout.sum(0)
    dh1 = (dout @ w6) * (h1 > 0)
    dw5, db5 = dh1.T @ h0, dh1.sum(0)
    dh0 = dh1 @ w5
    dy4 = np.repeat(dh0[:, None, :] / y4.shape[1], y4.shape[1], axis=1)
    return dy4, dw5, db5, dw6, db6


def bf16(a):
    """Round float values to bfloat16 (round to nearest even), as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)
