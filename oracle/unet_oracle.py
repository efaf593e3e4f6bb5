"""CPU oracle of the pressure-guess network -- test infrastructure only.

The reference (TURBINS) has no learned component: its Poisson solve starts from
the previous pressure (Solver.c:84).  This module restates, in numpy FP64, the
network the GPU library trains and runs (turbins_gb300/csrc/k_net.cu):

    a0 = relu(conv_in x0)        a1 = relu(conv1 pool a0)   a2 = relu(conv2 pool a1)
    a3 = relu(conv3 pool a2)     b3 = relu(conv3b a3)
    s2 = relu(up(conv_up2 b3) + a2)   b2 = relu(conv2b s2)
    s1 = relu(up(conv_up1 b2) + a1)   b1 = relu(conv1b s1)
    s0 = relu(up(conv_up0 b1) + a0)   b0 = relu(conv0b s0)
    out = head . b0 + hb

with 3x3x3 zero-padded convolutions out[v] = sum_tap W[tap] x[v + off(tap)],
tap = (dz*3 + dy)*3 + dx and off = (dx-1, dy-1, dz-1), 2x2x2 average pooling and
nearest upsampling.  With ``bf16=True`` every stored activation, gradient and
weight is rounded to bfloat16 (round to nearest even) where the GPU stores
one, so GPU and oracle differ only by accumulation order; with ``bf16=False``
it is plain FP64 (used to check the backward pass by finite differences).

Arrays are channel-major [C, Z, Y, X]; parameters are one flat FP32/FP64
vector in the library's order: per layer W[27][cout][cin] then b[cout], then
the 16 head weights and the head bias.
"""
from __future__ import annotations

import numpy as np

LAYERS = [(16, 16, 0), (16, 32, 1), (32, 64, 2), (64, 128, 3), (128, 128, 3), (128, 64, 3),
          (64, 64, 2), (64, 32, 2), (32, 32, 1), (32, 16, 1), (16, 16, 0)]


def bf16_round(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def param_layout():
    """(offset of W, offset of b) per layer, head weight and bias offsets, total."""
    offs, off = [], 0
    for cin, cout, _ in LAYERS:
        w = off
        off += 27 * cin * cout
        offs.append((w, off))
        off += cout
    return offs, off, off + 16, off + 17


def unpack(p):
    offs, hw, hb, n = param_layout()
    assert p.size == n
    Ws, bs = [], []
    for (cin, cout, _), (w, b) in zip(LAYERS, offs):
        Ws.append(p[w:w + 27 * cin * cout].reshape(27, cout, cin).astype(np.float64))
        bs.append(p[b:b + cout].astype(np.float64))
    return Ws, bs, p[hw:hw + 16].astype(np.float64), float(p[hb])


def conv3(x, W, b=None):
    C, Z, Y, X = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1)))
    out = np.zeros((W.shape[1], Z, Y, X))
    for t in range(27):
        dx, dy, dz = t % 3, (t // 3) % 3, t // 9
        out += np.einsum("oc,czyx->ozyx", W[t], xp[:, dz:dz + Z, dy:dy + Y, dx:dx + X], optimize=True)
    if b is not None:
        out += b[:, None, None, None]
    return out


def conv3_dgrad(dy, W):
    """d/dx of sum(dy * conv3(x, W))."""
    C, Z, Y, X = dy.shape
    dp = np.pad(dy, ((0, 0), (1, 1), (1, 1), (1, 1)))
    out = np.zeros((W.shape[2], Z, Y, X))
    for t in range(27):
        dx, dyy, dz = t % 3, (t // 3) % 3, t // 9
        out += np.einsum("oc,ozyx->czyx", W[t], dp[:, 2 - dz:2 - dz + Z, 2 - dyy:2 - dyy + Y, 2 - dx:2 - dx + X],
                         optimize=True)
    return out


def conv3_wgrad(x, dy):
    """d/dW of sum(dy * conv3(x, W)) as [27][cout][cin]."""
    C, Z, Y, X = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1)))
    g = np.zeros((27, dy.shape[0], C))
    for t in range(27):
        dx, dyy, dz = t % 3, (t // 3) % 3, t // 9
        g[t] = np.einsum("ozyx,czyx->oc", dy, xp[:, dz:dz + Z, dyy:dyy + Y, dx:dx + X], optimize=True)
    return g


def pool(a):
    C, Z, Y, X = a.shape
    return a.reshape(C, Z // 2, 2, Y // 2, 2, X // 2, 2).mean(axis=(2, 4, 6))


def up(c):
    return c.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def down_sum(d):
    C, Z, Y, X = d.shape
    return d.reshape(C, Z // 2, 2, Y // 2, 2, X // 2, 2).sum(axis=(2, 4, 6))


class UNet:
    def __init__(self, params, bf16=True):
        self.r = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
        self.Ws, self.bs, self.hw, self.hb = unpack(np.asarray(params))
        self.Wq = [self.r(W) for W in self.Ws]

    def _conv(self, l, x, relu=True):
        z = conv3(x, self.Wq[l], self.bs[l])
        return self.r(np.maximum(z, 0.0) if relu else z)

    def forward(self, in3):
        """in3: [3, Z, Y, X] -> out [Z, Y, X]; keeps the activations."""
        r = self.r
        x0 = np.zeros((16,) + in3.shape[1:])
        x0[:3] = r(in3)
        A = {"x0": x0}
        A["a0"] = self._conv(0, x0)
        A["p0"] = r(pool(A["a0"]))
        A["a1"] = self._conv(1, A["p0"])
        A["p1"] = r(pool(A["a1"]))
        A["a2"] = self._conv(2, A["p1"])
        A["p2"] = r(pool(A["a2"]))
        A["a3"] = self._conv(3, A["p2"])
        A["b3"] = self._conv(4, A["a3"])
        A["c2"] = self._conv(5, A["b3"], relu=False)
        A["s2"] = r(np.maximum(up(A["c2"]) + A["a2"], 0.0))
        A["b2"] = self._conv(6, A["s2"])
        A["c1"] = self._conv(7, A["b2"], relu=False)
        A["s1"] = r(np.maximum(up(A["c1"]) + A["a1"], 0.0))
        A["b1"] = self._conv(8, A["s1"])
        A["c0"] = self._conv(9, A["b1"], relu=False)
        A["s0"] = r(np.maximum(up(A["c0"]) + A["a0"], 0.0))
        A["b0"] = self._conv(10, A["s0"])
        self.A = A
        return np.einsum("c,czyx->zyx", self.hw, A["b0"]) + self.hb

    def backward(self, gout):
        """Gradients of sum(gout * out) for the last forward, as a flat vector."""
        r, A, Wq = self.r, self.A, self.Wq
        gW, gb = [None] * 11, [None] * 11

        def wg(l, x, d):
            gW[l] = conv3_wgrad(x, d)
            gb[l] = d.sum(axis=(1, 2, 3))

        ghw = np.einsum("czyx,zyx->c", A["b0"], gout)
        ghb = gout.sum()
        dz0b = r(self.hw[:, None, None, None] * gout[None] * (A["b0"] > 0))
        wg(10, A["s0"], dz0b)
        dzs0 = r(conv3_dgrad(dz0b, Wq[10]) * (A["s0"] > 0))
        dc0 = r(down_sum(dzs0))
        wg(9, A["b1"], dc0)
        dz1b = r(conv3_dgrad(dc0, Wq[9]) * (A["b1"] > 0))
        wg(8, A["s1"], dz1b)
        dzs1 = r(conv3_dgrad(dz1b, Wq[8]) * (A["s1"] > 0))
        dc1 = r(down_sum(dzs1))
        wg(7, A["b2"], dc1)
        dz2b = r(conv3_dgrad(dc1, Wq[7]) * (A["b2"] > 0))
        wg(6, A["s2"], dz2b)
        dzs2 = r(conv3_dgrad(dz2b, Wq[6]) * (A["s2"] > 0))
        dc2 = r(down_sum(dzs2))
        wg(5, A["b3"], dc2)
        dz3b = r(conv3_dgrad(dc2, Wq[5]) * (A["b3"] > 0))
        wg(4, A["a3"], dz3b)
        dz3 = r(conv3_dgrad(dz3b, Wq[4]) * (A["a3"] > 0))
        wg(3, A["p2"], dz3)
        dp2 = r(conv3_dgrad(dz3, Wq[3]))
        dz2 = r((dzs2 + up(dp2) * 0.125) * (A["a2"] > 0))
        wg(2, A["p1"], dz2)
        dp1 = r(conv3_dgrad(dz2, Wq[2]))
        dz1 = r((dzs1 + up(dp1) * 0.125) * (A["a1"] > 0))
        wg(1, A["p0"], dz1)
        dp0 = r(conv3_dgrad(dz1, Wq[1]))
        dz0 = r((dzs0 + up(dp0) * 0.125) * (A["a0"] > 0))
        wg(0, A["x0"], dz0)
        out = []
        for l in range(11):
            out.append(gW[l].ravel())
            out.append(gb[l])
        out.append(ghw)
        out.append(np.array([ghb]))
        return np.concatenate(out)


def init_params(seed):
    """He-normal convolution weights, zero biases, small head (numpy RNG; the
    library's own initialiser uses another generator)."""
    rng = np.random.default_rng(seed)
    offs, hw, hb, n = param_layout()
    p = np.zeros(n, dtype=np.float32)
    for (cin, cout, _), (w, b) in zip(LAYERS, offs):
        p[w:w + 27 * cin * cout] = rng.normal(0.0, np.sqrt(2.0 / (27 * cin)), 27 * cin * cout)
        p[b:b + cout] = rng.normal(0.0, 0.05, cout)
    p[hw:hw + 16] = rng.normal(0.0, 0.2, 16)
    p[hb] = 0.01
    return p


def to_blocked(a):
    """[C, Z, Y, X] -> the library's channel-blocked [C/8][Z][Y][X][8]."""
    C, Z, Y, X = a.shape
    return np.ascontiguousarray(a.reshape(C // 8, 8, Z, Y, X).transpose(0, 2, 3, 4, 1))


def from_blocked(b, C):
    nb, Z, Y, X, _ = b.shape
    return np.ascontiguousarray(b.transpose(0, 4, 1, 2, 3).reshape(C, Z, Y, X))


class Adam:
    """Adam (Kingma & Ba 2015) on the flat FP32 parameter vector, in float64:
    m = b1 m + (1 - b1) g, v = b2 v + (1 - b2) g^2,
    p -= lr (m / (1 - b1^t)) / (sqrt(v / (1 - b2^t)) + eps), with the
    library's constants b1 = 0.9, b2 = 0.999, eps = 1e-8 and the step count t
    restarting at 1 after new parameters are loaded."""

    def __init__(self, n, b1=0.9, b2=0.999, eps=1e-8):
        self.m = np.zeros(n)
        self.v = np.zeros(n)
        self.t = 0
        self.b1, self.b2, self.eps = b1, b2, eps

    def step(self, p, g, lr):
        self.t += 1
        g = np.asarray(g, dtype=np.float64)
        self.m = self.b1 * self.m + (1.0 - self.b1) * g
        self.v = self.b2 * self.v + (1.0 - self.b2) * g * g
        c1 = 1.0 - self.b1 ** self.t
        c2 = 1.0 - self.b2 ** self.t
        return np.asarray(p, dtype=np.float64) - lr * (self.m / c1) / (np.sqrt(self.v / c2) + self.eps)
