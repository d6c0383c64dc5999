"""ORACLE — test infrastructure, not product code.

numpy restatement of the warm-start network of gfmd_warmstart.cu (forward,
mean-squared-error loss, backward) in the same parameter layout: per layer
W[cout][9][cin] (tap = 3 (dy+1) + (dx+1)), then b[cout].  With
``bf16=True`` the convolution operands are rounded to BF16 (round to
nearest even) where the GPU kernels stage them — inputs and filters in the
forward and data-gradient convolutions, inputs and output gradients in the
weight gradient — and accumulated in FP64; tensors between layers are FP32
as on the GPU.  With ``bf16=False`` everything is FP64 (for the
finite-difference check of the backward pass itself).  Only tests/ import
this module.
"""
from __future__ import annotations

import numpy as np


def to_bf16(a):
    """Round to BF16 (nearest even) and return as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    b = a32.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


class Net:
    def __init__(self, in_ch, out_ch, base, bf16=True):
        C, C2 = base, 2 * base
        self.io = [(in_ch, C), (C, C), (C, C2), (C2, C2), (C2, C2), (C2, C2), (C2, C), (C, C), (C, out_ch)]
        self.offs = []
        off = 0
        for ci, co in self.io:
            self.offs.append((off, off + co * 9 * ci))
            off += co * 9 * ci + co
        self.nparam = off
        self.bf16 = bf16

    def _r(self, a):
        return to_bf16(a) if self.bf16 else np.asarray(a, np.float64)

    def _s(self, a):
        """Storage rounding of a tensor between layers (FP32 on the GPU)."""
        return np.asarray(a, np.float32).astype(np.float64) if self.bf16 else a

    def layer(self, w, i):
        ci, co = self.io[i]
        a, b = self.offs[i]
        return w[a:b].reshape(co, 9, ci), w[b:b + co]

    @staticmethod
    def _shift(x, t, sign=1):
        dy, dx = t // 3 - 1, t % 3 - 1
        # out[p] = x[p + sign * off(t)] (periodic)
        return np.roll(x, shift=(-sign * dy, -sign * dx), axis=(1, 2))

    def conv(self, x, W, b, relu):
        xs, Ws = self._r(x), self._r(W)
        y = np.zeros(x.shape[:3] + (W.shape[0],))
        for t in range(9):
            y += self._shift(xs, t) @ Ws[:, t, :].T
        y += b
        if relu:
            y = np.maximum(y, 0.0)
        return self._s(y)

    def conv_bwd(self, x, W, g):
        """(dX, dW, db) of y = conv(x, W) + b for output gradient g."""
        gs, Ws, xs = self._r(g), self._r(W), self._r(x)
        dx = np.zeros(x.shape)
        dW = np.zeros(W.shape)
        for t in range(9):
            dx += self._shift(gs, t, -1) @ Ws[:, t, :]
            xt = self._shift(xs, t)
            dW[:, t, :] = np.einsum("nhwo,nhwi->oi", gs, xt)
        db = np.asarray(g, np.float64).sum(axis=(0, 1, 2))
        return self._s(dx), dW, db

    @staticmethod
    def pool(x):
        return 0.25 * (x[:, 0::2, 0::2] + x[:, 1::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 1::2])

    @staticmethod
    def pool_bwd(g):
        return 0.25 * np.repeat(np.repeat(g, 2, axis=1), 2, axis=2)

    @staticmethod
    def up(x):
        return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)

    @staticmethod
    def up_bwd(g):
        return g[:, 0::2, 0::2] + g[:, 1::2, 0::2] + g[:, 0::2, 1::2] + g[:, 1::2, 1::2]

    def forward(self, w, x):
        L = lambda i: self.layer(w, i)  # noqa: E731
        A = {"x": np.asarray(x, np.float64)}
        A["a1"] = self.conv(A["x"], *L(0), True)
        A["a2"] = self.conv(A["a1"], *L(1), True)
        A["p1"] = self._s(self.pool(A["a2"]))
        A["a3"] = self.conv(A["p1"], *L(2), True)
        A["p2"] = self._s(self.pool(A["a3"]))
        A["a4"] = self.conv(A["p2"], *L(3), True)
        A["p3"] = self._s(self.pool(A["a4"]))
        A["a5"] = self.conv(A["p3"], *L(4), True)
        A["s2"] = self._s(self.up(A["a5"]) + A["a4"])
        A["a6"] = self.conv(A["s2"], *L(5), True)
        A["s1"] = self._s(self.up(A["a6"]) + A["a3"])
        A["a7"] = self.conv(A["s1"], *L(6), True)
        A["s0"] = self._s(self.up(A["a7"]) + A["a2"])
        A["a8"] = self.conv(A["s0"], *L(7), True)
        A["y"] = self.conv(A["a8"], *L(8), False)
        return A

    def loss_grad(self, w, x, target):
        A = self.forward(w, x)
        d = A["y"] - target
        loss = float((d * d).mean())
        gy = self._s(2.0 * d / d.size)
        grad = np.zeros(self.nparam)

        def put(i, dW, db):
            a, b = self.offs[i]
            grad[a:b] = dW.ravel()
            grad[b:b + db.size] = db

        relu = lambda g, a: np.where(a > 0, g, 0.0)  # noqa: E731
        gx, dW, db = self.conv_bwd(A["a8"], self.layer(w, 8)[0], gy); put(8, dW, db)
        g = relu(gx, A["a8"])
        gs0, dW, db = self.conv_bwd(A["s0"], self.layer(w, 7)[0], g); put(7, dW, db)
        g = relu(self._s(self.up_bwd(gs0)), A["a7"])
        gs1, dW, db = self.conv_bwd(A["s1"], self.layer(w, 6)[0], g); put(6, dW, db)
        g = relu(self._s(self.up_bwd(gs1)), A["a6"])
        gs2, dW, db = self.conv_bwd(A["s2"], self.layer(w, 5)[0], g); put(5, dW, db)
        g = relu(self._s(self.up_bwd(gs2)), A["a5"])
        gp3, dW, db = self.conv_bwd(A["p3"], self.layer(w, 4)[0], g); put(4, dW, db)
        g = relu(self._s(self.pool_bwd(gp3) + gs2), A["a4"])
        gp2, dW, db = self.conv_bwd(A["p2"], self.layer(w, 3)[0], g); put(3, dW, db)
        g = relu(self._s(self.pool_bwd(gp2) + gs1), A["a3"])
        gp1, dW, db = self.conv_bwd(A["p1"], self.layer(w, 2)[0], g); put(2, dW, db)
        g = relu(self._s(self.pool_bwd(gp1) + gs0), A["a2"])
        ga1, dW, db = self.conv_bwd(A["a1"], self.layer(w, 1)[0], g); put(1, dW, db)
        g = relu(ga1, A["a1"])
        _, dW, db = self.conv_bwd(A["x"], self.layer(w, 0)[0], g); put(0, dW, db)
        return loss, grad, A["y"]


def he_init(net, seed):
    """The GPU's initial weights: He-uniform from a SplitMix64 stream."""
    w = np.zeros(net.nparam, np.float32)
    st = seed
    M = (1 << 64) - 1
    for i, (ci, co) in enumerate(net.io):
        a, b = net.offs[i]
        lim = float(np.sqrt(np.float32(6.0) / np.float32(9.0 * ci)))  # FP32 sqrt, used in FP64
        for k in range(co * 9 * ci):
            z = (st + 0x9E3779B97F4A7C15) & M
            st = z
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
            z ^= z >> 31
            st_out = z
            u = (st_out >> 11) * 2.0 ** -53
            w[a + k] = np.float32((2.0 * u - 1.0) * lim)
            st = st_out
    return w
