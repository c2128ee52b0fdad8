"""The schedule network on the device, driven through the C ABI.

Architecture (64^3 bf16 input, channels last): four 3x3x3 convolutions with
stride 2 and padding 1 (1 -> 16 -> 32 -> 64 -> 64 channels, 64^3 -> 4^3),
bias + ReLU after each; global average pool; MLP 64 -> 64 (ReLU) -> 64;
sigmoid: the predicted saturation at 64 radii.  Convolutions run on the
library's tcgen05 implicit-GEMM kernels (bf16 operands, fp32 accumulate),
forward and backward; the head, the loss and Adam are fp32 kernels.

All parameters live in one flat fp32 vector (layout in LAYERS / HEAD), the
Adam moments beside it; ``save`` / ``load`` keep all three (and the step
count) so training resumes where it stopped.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from .._lib import check, lib

# (input side, c_in, c_out) of the four convolutions
LAYERS = [(64, 1, 16), (32, 16, 32), (16, 32, 64), (8, 64, 64)]
HEAD = 64
N_RADII = 64
KBK = 64


def _kpad(k: int) -> int:
    return (k + KBK - 1) // KBK * KBK


def param_layout():
    """[(name, shape)] in flat-vector order."""
    out = []
    for i, (_, cin, cout) in enumerate(LAYERS, 1):
        out.append((f"w{i}", (cout, cin, 27)))
        out.append((f"b{i}", (cout,)))
    out += [("w5", (HEAD, HEAD)), ("b5", (HEAD,)), ("w6", (N_RADII, HEAD)), ("b6", (N_RADII,))]
    return out


def _declare(L):
    P, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    sig = {
        "pmg_cnn_pack_weights": [P, i32, i32, P, P, P],
        "pmg_cnn_conv_fwd": [P, P, P, P, i32, i32, i32, i32, P, P],
        "pmg_cnn_conv_dgrad": [P, P, P, P, i32, i32, i32, i32, P, P],
        "pmg_cnn_conv_wgrad": [P, P, P, P, P, i32, i32, i32, i32, P, P],
        "pmg_cnn_head": [P, P, i32, P, P, P, P, P, P],
        "pmg_cnn_adam": [P, P, P, P, i64, f64, f64, f64, f64, i64, f64, P],
        "pmg_cnn_downsample": [P, P, P, f64, P, P],
        "pmg_cnn_check": [P, P],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int


_declared = False


def L():
    global _declared
    lb = lib()
    if not _declared:
        _declare(lb)
        _declared = True
    return lb


def _p(t: torch.Tensor | None):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class ScheduleNet:
    """Parameters, optimizer state and the forward / backward passes."""

    def __init__(self, seed: int = 0, device="cuda"):
        self.device = torch.device(device)
        self.layout = param_layout()
        self.offsets = {}
        off = 0
        for name, shape in self.layout:
            self.offsets[name] = (off, shape)
            off += int(np.prod(shape))
        self.n_params = off
        self.params = torch.zeros(off, dtype=torch.float32, device=self.device)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._init(seed)
        self.wk, self.wkt, self.dwbuf = [], [], []
        for (_, cin, cout) in LAYERS:
            self.wk.append(torch.zeros(cout * _kpad(27 * cin), dtype=torch.bfloat16, device=self.device))
            self.wkt.append(torch.zeros(cin * _kpad(27 * cout), dtype=torch.bfloat16, device=self.device)
                            if cin >= 16 else None)
            self.dwbuf.append(torch.zeros(27 * cin * cout, dtype=torch.float32, device=self.device))
        self._acts = {}
        self.pack()

    def view(self, name, t=None):
        off, shape = self.offsets[name]
        t = self.params if t is None else t
        return t[off:off + int(np.prod(shape))].view(*shape)

    def _init(self, seed):
        g = torch.Generator(device="cpu")
        g.manual_seed(seed)
        for name, shape in self.layout:
            if name.startswith("w"):
                fan_in = shape[1] * (shape[2] if len(shape) == 3 else 1)
                w = torch.randn(shape, generator=g) * math.sqrt(2.0 / fan_in)
                self.view(name).copy_(w.reshape(-1).view(*shape))
        # start the output near the middle of the saturation range
        self.view("b6").fill_(0.0)

    def pack(self):
        """bf16 GEMM operands of the convolution weights from the fp32 master."""
        st = _stream()
        for i, (_, cin, cout) in enumerate(LAYERS, 1):
            check(L().pmg_cnn_pack_weights(_p(self.view(f"w{i}")), cin, cout, _p(self.wk[i - 1]),
                                           _p(self.wkt[i - 1]), st), "cnn pack")

    def _buffers(self, batch):
        if batch not in self._acts:
            a = {"x": None}
            for i, (d, cin, cout) in enumerate(LAYERS, 1):
                do = (d + 1) // 2
                a[f"y{i}"] = torch.empty(batch * do ** 3 * cout, dtype=torch.bfloat16, device=self.device)
                a[f"dz{i}"] = torch.empty_like(a[f"y{i}"])
            a["pred"] = torch.empty(batch * N_RADII, dtype=torch.float32, device=self.device)
            a["loss"] = torch.zeros(1, dtype=torch.float32, device=self.device)
            self._acts[batch] = a
        return self._acts[batch]

    def forward(self, x: torch.Tensor, target: torch.Tensor | None = None):
        """x: bf16 [batch, 64, 64, 64] (or [batch, 64^3]); returns the fp32
        predictions [batch, 64] (and, with a target, leaves the loss and the
        head's gradients for backward)."""
        batch = x.shape[0]
        a = self._buffers(batch)
        st = _stream()
        h = x.contiguous()
        for i, (d, cin, cout) in enumerate(LAYERS, 1):
            check(L().pmg_cnn_conv_fwd(_p(h), _p(self.wk[i - 1]), _p(self.view(f"b{i}")), _p(a[f"y{i}"]), batch, d,
                                       cin, cout, _p(self.err), st), "cnn conv forward")
            h = a[f"y{i}"]
        head = self.params[self.offsets["w5"][0]:]
        if target is not None:
            a["loss"].zero_()
            self.grads.zero_()
            ghead = self.grads[self.offsets["w5"][0]:]
            check(L().pmg_cnn_head(_p(h), _p(head), batch, _p(target.contiguous()), _p(a["pred"]), _p(a["loss"]),
                                   _p(ghead), _p(a["dz4"]), st), "cnn head")
        else:
            check(L().pmg_cnn_head(_p(h), _p(head), batch, None, _p(a["pred"]), None, None, None, st), "cnn head")
        return a["pred"].view(batch, N_RADII)

    def backward(self, x: torch.Tensor):
        """Gradients of the loss of the last forward(x, target) into self.grads."""
        batch = x.shape[0]
        a = self._buffers(batch)
        st = _stream()
        ins = [x.contiguous(), a["y1"], a["y2"], a["y3"]]
        for i in range(len(LAYERS), 0, -1):
            d, cin, cout = LAYERS[i - 1]
            check(L().pmg_cnn_conv_wgrad(_p(ins[i - 1]), _p(a[f"dz{i}"]), _p(self.dwbuf[i - 1]),
                                         _p(self.view(f"w{i}", self.grads)), _p(self.view(f"b{i}", self.grads)),
                                         batch, d, cin, cout, _p(self.err), st), "cnn conv wgrad")
            if i > 1:
                check(L().pmg_cnn_conv_dgrad(_p(a[f"dz{i}"]), _p(self.wkt[i - 1]), _p(ins[i - 1]),
                                             _p(a[f"dz{i - 1}"]), batch, d, cin, cout, _p(self.err), st),
                      "cnn conv dgrad")

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0):
        self.step += 1
        check(L().pmg_cnn_adam(_p(self.params), _p(self.grads), _p(self.m), _p(self.v), self.n_params, lr, b1, b2,
                               eps, self.step, weight_decay, _stream()), "cnn adam")
        self.pack()

    def train_step(self, x, target, lr=1e-3):
        self.forward(x, target)
        self.backward(x)
        self.adam_step(lr=lr)
        return self._buffers(x.shape[0])["loss"]

    def check_status(self):
        check(L().pmg_cnn_check(_p(self.err), _stream()), "cnn")

    def predict(self, x: torch.Tensor) -> torch.Tensor:
        with torch.no_grad():
            return self.forward(x).clone()

    # ---- persistence ------------------------------------------------------------
    def state(self):
        return {"params": self.params.cpu(), "m": self.m.cpu(), "v": self.v.cpu(), "step": self.step,
                "layout": self.layout}

    def save(self, path):
        torch.save(self.state(), path)

    def load_state(self, st):
        if [tuple(x) for x in st["layout"]] != [(n, tuple(s)) for n, s in self.layout]:
            raise ValueError("saved network has a different layout")
        self.params.copy_(st["params"].to(self.device))
        self.m.copy_(st["m"].to(self.device))
        self.v.copy_(st["v"].to(self.device))
        self.step = int(st["step"])
        self.pack()

    @classmethod
    def load(cls, path, device="cuda"):
        net = cls(device=device)
        net.load_state(torch.load(path, map_location="cpu", weights_only=False))
        return net
