"""Properties of the FP64 Poisson restatement (CPU only): the operator is
symmetric positive definite on the value-block cells, the V-cycle is a symmetric
positive definite preconditioner, MG-PCG reaches 1e-6, and the seeded face
coefficients lie in [0.5, 2]."""
from __future__ import annotations

import numpy as np
import pytest

from msbg_gb300 import workloads as W


@pytest.fixture(scope="module")
def prob(port):
    res, bs = 96, 16
    pts = W.sphere_cloud(res, 4, 2000, seed=W.workload_seed(3, 2), radius_range=(0.08, 0.15))
    g = port.grid(res, res, res, bs, port.F32)
    cnt, valid, nv = port.mark_blocks(g, pts, 4.0)
    bids = np.nonzero(cnt > 0)[0].astype(np.int64)
    return port.PoissonProblem(bids, (g.nbx, g.nby, g.nbz), bs, seed=7)


def test_coefficients_range(prob):
    a = prob.act > 0
    for c in (prob.cx, prob.cy, prob.cz):
        assert c[a].min() >= 0.5 and c[a].max() <= 2.0
    assert np.all(prob.d[a] >= 3.0) and np.all(prob.d[a] <= 12.0)


def test_operator_spd(prob):
    rng = np.random.default_rng(0)
    x = rng.standard_normal(prob.act.shape) * prob.act
    y = rng.standard_normal(prob.act.shape) * prob.act
    assert abs(np.sum(prob.apply(x) * y) - np.sum(x * prob.apply(y))) < 1e-9 * abs(np.sum(prob.apply(x) * y))
    assert np.sum(prob.apply(x) * x) > 0


@pytest.mark.parametrize("pre,post,k", [(2, 2, 1), (1, 1, 3)])
def test_vcycle_spd_params(port, prob, pre, post, k):
    """Pre- and post-smoother are adjoint for every pass/in-tile-sweep setting."""
    p2 = port.PoissonProblem(prob.bids, prob.nb, prob.bs, seed=7, pre=pre, post=post, tile_iters=k)
    rng = np.random.default_rng(11)
    a = rng.standard_normal(p2.act.shape) * p2.act
    b = rng.standard_normal(p2.act.shape) * p2.act
    ma, _ = p2.vcycle(a)
    mb, _ = p2.vcycle(b)
    assert abs(np.sum(ma * b) - np.sum(a * mb)) < 1e-8 * abs(np.sum(ma * b))
    assert np.sum(ma * a) > 0


def test_tile_smoother_reduces_energy_bs32(port):
    """bs32 levels smooth in 16^3 tiles (4 of each colour per block): each pass
    lowers the A-norm of the error."""
    res, bs = 128, 32
    pts = W.sphere_cloud(res, 3, 2000, seed=W.workload_seed(3, 3), radius_range=(0.1, 0.2))
    g = port.grid(res, res, res, bs, port.F32)
    cnt, valid, nv = port.mark_blocks(g, pts, 4.0)
    bids = np.nonzero(cnt > 0)[0].astype(np.int64)
    p = port.PoissonProblem(bids, (g.nbx, g.nby, g.nbz), bs, seed=9)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(p.act.shape) * p.act
    xs, it, rel = p.solve(b, 1e-10, max_iter=100)
    assert rel <= 1e-10
    x = np.zeros_like(b)
    energy = []
    for _ in range(3):
        x = p.smooth(x, b, 1)
        e = x - xs
        energy.append(float(np.sum(e * p.apply(e))))
    assert energy[0] > energy[1] > energy[2]


def test_vcycle_spd(prob):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(prob.act.shape) * prob.act
    b = rng.standard_normal(prob.act.shape) * prob.act
    ma, _ = prob.vcycle(a)
    mb, _ = prob.vcycle(b)
    assert abs(np.sum(ma * b) - np.sum(a * mb)) < 1e-8 * abs(np.sum(ma * b))
    assert np.sum(ma * a) > 0


def test_mgpcg_converges(prob):
    rng = np.random.default_rng(2)
    b = rng.standard_normal(prob.act.shape) * prob.act
    x, it, rel = prob.solve(b, 1e-6)
    assert rel <= 1e-6 and it < 40
    assert prob.rel_residual(x, b) <= 1e-6
