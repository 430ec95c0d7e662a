"""The CPU restatement of the learned warm start (oracle/warmnet.py): its backward
pass agrees with finite differences of its forward pass (CPU only)."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import warmnet as WN  # noqa: E402


def _operator(n, rng):
    cx, cy, cz = (rng.uniform(0.5, 2.0, (n, n, n)) for _ in range(3))

    def apply(x):
        y = np.zeros_like(x)
        d = np.zeros_like(x)
        # faces between (z,y,x-1)-(z,y,x) carry cx[z,y,x], and so on
        for arr, ax in ((cx, 2), (cy, 1), (cz, 0)):
            sl_hi = [slice(None)] * 3
            sl_lo = [slice(None)] * 3
            sl_hi[ax] = slice(1, None)
            sl_lo[ax] = slice(0, -1)
            c = arr[tuple(sl_hi)]
            y[tuple(sl_hi)] -= c * x[tuple(sl_lo)]
            y[tuple(sl_lo)] -= c * x[tuple(sl_hi)]
            d[tuple(sl_hi)] += c
            d[tuple(sl_lo)] += c
        return y + (d + 1.0) * x

    return apply


@pytest.fixture(scope="module")
def problem():
    rng = np.random.default_rng(5)
    n = 8
    mask0 = np.ones((n, n, n))
    a0 = _operator(n, rng)
    b0 = rng.standard_normal((n, n, n))
    xs = rng.standard_normal((n, n, n)) * 0.3
    d1 = rng.uniform(3.0, 9.0, (n // 2,) * 3)
    net = WN.WarmNet.init(17)
    return net, b0, xs, mask0, a0, d1


def test_bf16_round_ties_to_even():
    v = np.array([1.0, 1.00390625, 1.01171875, -2.5], np.float32)  # 1+2^-8 is a tie
    r = WN.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.015625) and r[3] == -2.5


@pytest.mark.parametrize("loss", ["coarse", "residual"])
def test_gradients_match_finite_differences(problem, loss):
    net, b0, xs, mask0, a0, d1 = problem
    L, gW, gc, _ = WN.loss_and_grads(net, b0, xs, mask0, a0, d1, loss=loss)
    assert np.isfinite(L) and L > 0
    rng = np.random.default_rng(3)
    # finite differences on the (bf16-rounded) weights: perturb the rounded value by a
    # step that survives rounding, i.e. compare against the analytic gradient of the
    # rounded weights with central differences on float64 copies
    for l in (0, 1, 3):
        for _ in range(4):
            t = rng.integers(27)
            i = rng.integers(WN.CH[l])
            o = rng.integers(WN.CH[l + 1])
            h = 1e-3

            def lossw(delta):
                W = [w.copy() for w in net.W]
                base = WN.bf16_round(W[l])
                Wd = [WN.bf16_round(w) for w in W]
                Wd[l] = base.copy()
                Wd[l][t, i, o] += delta
                n2 = WN.WarmNet(W, net.c)
                # bypass rounding for the perturbed copy
                orig = WN.bf16_round
                WN.bf16_round = lambda w, _m={id(x): y for x, y in zip(W, Wd)}: _m.get(id(w), orig(w))
                try:
                    return WN.loss_and_grads(n2, b0, xs, mask0, a0, d1, loss=loss)[0]
                finally:
                    WN.bf16_round = orig

            fd = (lossw(h) - lossw(-h)) / (2 * h)
            assert abs(fd - gW[l][t, i, o]) <= 1e-4 * max(1.0, abs(fd)), (l, t, i, o, fd, gW[l][t, i, o])
    for l in (0, 2):
        o = rng.integers(WN.CH[l + 1])
        h = 1e-7
        cp = [c.copy() for c in net.c]
        cm = [c.copy() for c in net.c]
        cp[l] = cp[l].astype(np.float64)
        cm[l] = cm[l].astype(np.float64)
        cp[l][o] += h
        cm[l][o] -= h
        fd = (WN.loss_and_grads(WN.WarmNet(net.W, cp), b0, xs, mask0, a0, d1, loss=loss)[0]
              - WN.loss_and_grads(WN.WarmNet(net.W, cm), b0, xs, mask0, a0, d1, loss=loss)[0]) / (2 * h)
        assert abs(fd - gc[l][o]) <= 1e-4 * max(1.0, abs(fd))
