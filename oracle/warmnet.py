"""CPU restatement (numpy, float64) of the learned warm start -- test infrastructure only.

The reference has no learned component; this file restates the network that the
GPU library implements (msbg_gb300/csrc/warmnet.cu) so the GPU forward pass, loss
and gradients can be checked on small dense volumes.

Network (on the level-1 cells of the multigrid hierarchy, i.e. the value blocks
with their edge halved, dense here with an activity mask):

    in  = [ b1 / s,  d1 / dbar - 1 ]          b1 = sum of the 8 level-0 children of b,
                                              d1 = level-1 diagonal, s = rms(b1) over
                                              active cells, dbar = mean(d1)
    h1  = relu(conv(in, W1) + c1)             conv: 3x3x3, zero outside active cells
    h2  = relu(conv(h1, W2) + c2)             channels 2 -> 16 -> 16 -> 16 -> 2
    h3  = relu(conv(h2, W3) + c3)
    o   = conv(h3, W4) + c4
    x1  = s * (o[0] + P2 avg2(o[1]))          avg2: mean over the 8 cells of a level-2
                                              parent, P2: back to every child
    x0  = P1 x1                               the level-1 value on each of its 8 children

Weights are rounded to BF16 before use (W[tap][cin][cout], tap = dx + 3 dy + 9 dz
with offsets -1..1); activations and accumulation are FP32 on the GPU, float64 here.
Losses: "residual" L = ||A0 (x0 - x*)||^2 / ||b||^2 with A0 the level-0 operator;
"coarse" L = ||x1 - avg1(x*)||^2 / ||avg1(x*)||^2 with avg1(x*) the mean of the 8
level-0 children of every level-1 cell (the warm start's best coarse value).
"""
from __future__ import annotations

import numpy as np

CH = (2, 16, 16, 16, 2)


def bf16_round(w: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(w, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def taps():
    return [(dx, dy, dz) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def shift(a: np.ndarray, dx: int, dy: int, dz: int) -> np.ndarray:
    """out[z, y, x] = a[z + dz, y + dy, x + dx] (zero outside); a is [z, y, x, C]."""
    out = np.zeros_like(a)
    nz, ny, nx = a.shape[:3]
    zs, ze = max(0, -dz), min(nz, nz - dz)
    ys, ye = max(0, -dy), min(ny, ny - dy)
    xs, xe = max(0, -dx), min(nx, nx - dx)
    out[zs:ze, ys:ye, xs:xe] = a[zs + dz:ze + dz, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv(a: np.ndarray, w: np.ndarray, bias: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """3x3x3 convolution of a [z, y, x, Cin] with w [27, Cin, Cout]; zero at inactive cells."""
    out = np.zeros(a.shape[:3] + (w.shape[2],))
    for t, (dx, dy, dz) in enumerate(taps()):
        out += shift(a, dx, dy, dz) @ w[t]
    return (out + bias) * mask[..., None]


def conv_backward(a: np.ndarray, w: np.ndarray, g: np.ndarray, mask: np.ndarray):
    """Gradients of conv w.r.t. input, weights and bias for upstream g [z, y, x, Cout]."""
    g = g * mask[..., None]
    ga = np.zeros_like(a)
    gw = np.zeros_like(w)
    for t, (dx, dy, dz) in enumerate(taps()):
        sa = shift(a, dx, dy, dz)
        gw[t] = sa.reshape(-1, a.shape[3]).T @ g.reshape(-1, g.shape[3])
        ga += shift(g @ w[t].T, -dx, -dy, -dz)
    gb = g.reshape(-1, g.shape[3]).sum(axis=0)
    return ga * mask[..., None], gw, gb


def avg2(v: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """Mean over the 8 cells of each 2x2x2 group (level-2 parent), back on every cell."""
    nz, ny, nx = v.shape
    m = (v * mask).reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2).sum(axis=(1, 3, 5)) / 8.0
    return np.repeat(np.repeat(np.repeat(m, 2, 0), 2, 1), 2, 2) * mask


def prolong(x1: np.ndarray) -> np.ndarray:
    return np.repeat(np.repeat(np.repeat(x1, 2, 0), 2, 1), 2, 2)


def restrict_sum(x0: np.ndarray) -> np.ndarray:
    nz, ny, nx = x0.shape
    return x0.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2).sum(axis=(1, 3, 5))


class WarmNet:
    """Weights W[l] ([27, Cin, Cout], float32 masters) and biases c[l]."""

    def __init__(self, weights, biases):
        self.W = [np.asarray(w, np.float32) for w in weights]
        self.c = [np.asarray(b) for b in biases]

    @staticmethod
    def init(seed: int) -> "WarmNet":
        rng = np.random.Generator(np.random.PCG64(seed))
        W, c = [], []
        for l in range(4):
            cin, cout = CH[l], CH[l + 1]
            std = np.sqrt(2.0 / (27 * cin)) * (0.5 if l == 3 else 1.0)
            W.append(rng.normal(0.0, std, (27, cin, cout)).astype(np.float32))
            c.append(np.zeros(cout, np.float32))
        return WarmNet(W, c)

    def forward(self, b1: np.ndarray, d1: np.ndarray, mask1: np.ndarray, act_bf16: bool = False):
        """Level-1 warm start x1 and the cache for backward.  act_bf16: every
        convolution reads its input activations rounded to BF16, as the tensor-core
        forward does (the backward pass, like the GPU's, uses the unrounded ones)."""
        act = mask1 > 0
        s = float(np.sqrt(np.mean(b1[act] ** 2))) if act.any() else 1.0
        s = s if s > 0 else 1.0
        dbar = float(np.mean(d1[act])) if act.any() else 1.0
        inp = np.stack([b1 / s, (d1 / dbar - 1.0)], axis=-1) * mask1[..., None]
        Wq = [bf16_round(w) for w in self.W]
        hs = [inp]
        for l in range(4):
            a = bf16_round(hs[-1]) if act_bf16 else hs[-1]
            h = conv(a, Wq[l], self.c[l].astype(np.float64), mask1)
            if l < 3:
                h = np.maximum(h, 0.0)
            hs.append(h)
        o = hs[-1]
        x1 = s * (o[..., 0] + avg2(o[..., 1], mask1)) * mask1
        return x1, (hs, Wq, s, mask1)

    def backward(self, gx1: np.ndarray, cache):
        """Gradients w.r.t. W (of the BF16-rounded weights) and c for upstream gx1."""
        hs, Wq, s, mask1 = cache
        g = np.zeros(hs[-1].shape)
        g[..., 0] = s * gx1 * mask1
        g[..., 1] = s * avg2(gx1 * mask1, mask1)
        gW, gc = [None] * 4, [None] * 4
        for l in range(3, -1, -1):
            if l < 3:
                g = g * (hs[l + 1] > 0)
            ga, gW[l], gc[l] = conv_backward(hs[l], Wq[l], g, mask1)
            g = ga
        return gW, gc


def loss_and_grads(net: WarmNet, b0, xstar0, mask0, apply_a0, d1, loss: str = "coarse", act_bf16: bool = False):
    """The loss and its gradients (dense level-0 arrays; apply_a0(x) applies the
    level-0 operator)."""
    mask1 = (restrict_sum(mask0.astype(np.float64)) > 0).astype(np.float64)
    b1 = restrict_sum(b0 * mask0)
    x1, cache = net.forward(b1, d1, mask1, act_bf16)
    x0 = prolong(x1) * mask0
    if loss == "residual":
        e = apply_a0(x0 - xstar0)
        bn = float(np.sum(b0 * b0))
        L = float(np.sum(e * e)) / bn
        gx0 = 2.0 * apply_a0(e) / bn
        gx1 = restrict_sum(gx0 * mask0)
    else:
        xbar = restrict_sum(xstar0 * mask0) / 8.0 * mask1
        dd = (x1 - xbar) * mask1
        den = float(np.sum(xbar * xbar))
        L = float(np.sum(dd * dd)) / den
        gx1 = 2.0 * dd / den
    gW, gc = net.backward(gx1, cache)
    return L, gW, gc, x0
