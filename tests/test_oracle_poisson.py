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
