"""Batched solves (segmented MG-PCG over independent volumes of one layout): every
volume reaches the tolerance, the batch solution equals the FP64 restatement's
solve, each volume takes the iterations it takes when solved alone, and the CUDA
graph path gives the same bits as the eager path."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

CH_X, CH_B = 1, 2
RES, BS = 128, 16          # 8^3 blocks, 8 volumes of 4^3 blocks (2 x 2 x 2)


def _layout(seed=3):
    """Volume v owns the inner blocks of its 4^3-block cell (a random subset of the
    2^3 centre blocks plus at least one), so volumes never touch."""
    rng = np.random.default_rng(seed)
    nb = RES // BS
    levels = np.ones((nb, nb, nb), np.int32)
    vol = np.full((nb, nb, nb), -1, np.int32)
    for v in range(8):
        ox, oy, oz = 4 * (v & 1), 4 * ((v >> 1) & 1), 4 * (v >> 2)
        m = rng.random((2, 2, 2)) < 0.7
        m[0, 0, 0] = True
        for k in range(8):
            x, y, z = k & 1, (k >> 1) & 1, k >> 2
            if m[z, y, x]:
                levels[oz + 1 + z, oy + 1 + y, ox + 1 + x] = 0
                vol[oz + 1 + z, oy + 1 + y, ox + 1 + x] = v
    return levels.reshape(-1), vol.reshape(-1)


@pytest.fixture(scope="module")
def batch(gpulib, port):
    G, P = gpulib, port
    levels, vol = _layout()
    g = G.MultiresSparseGrid(RES, RES, RES, BS, 2, G.F32)
    g.set_levels(levels)
    g.setRefinementMap(0.0)
    for ch in (CH_X, CH_B):
        g.channel_create(ch, G.F32)
    g.poisson_procedural_coefficients(777)
    g.batch_set_volumes(vol, 8)
    bids = g.active_blocks().astype(np.int64)
    prob = P.PoissonProblem(bids, (g.nbx, g.nby, g.nbz), BS, seed=777)
    yield G, P, g, prob, vol
    g.close()


def _rhs(prob, rng, scale_per_volume=None):
    b = np.where(prob.act > 0, rng.standard_normal(prob.act.shape), 0.0)
    return b


def test_batch_matches_fp64_solve(batch):
    G, P, g, prob, vol = batch
    rng = np.random.default_rng(1)
    b = _rhs(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(b), CH_B)
    g.fill(0.0, CH_X)
    its, ms, rel, tot = g.batch_mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=60)
    # convergence is confirmed on the true residual, so every volume meets the tolerance
    assert np.all(its >= 1) and np.all(rel <= 1e-6), (its, rel)
    assert np.all(ms > 0) and np.all(ms <= tot + 1e-3)
    x = prob.dense(g.payload(CH_X))
    xs, _, _ = prob.solve(b.astype(np.float64), 1e-9, 200)
    assert rel_l2(x, xs) < 1e-5


def test_volume_iterations_equal_solo_solves(batch):
    G, P, g, prob, vol = batch
    rng = np.random.default_rng(2)
    # volumes with very different right-hand-side scales converge independently
    b = _rhs(prob, rng)
    bpay = prob.payload(b)
    slot_vol = vol[prob.bids]
    bpay *= (10.0 ** (slot_vol % 4 - 2))[:, None]
    g.upload_payload(bpay.astype(np.float32), CH_B)
    g.fill(0.0, CH_X)
    its, ms, rel, tot = g.batch_mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=60)
    assert np.all(rel <= 1e-6)
    for v in range(8):
        solo = np.where((slot_vol == v)[:, None], bpay, 0.0).astype(np.float32)
        g.upload_payload(solo, CH_B)
        g.fill(0.0, CH_X)
        it_solo, rel_solo = g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=60)
        assert abs(int(its[v]) - it_solo) <= 1, (v, its[v], it_solo)


def test_graph_and_eager_paths_are_bit_identical(batch):
    G, P, g, prob, vol = batch
    rng = np.random.default_rng(3)
    b = _rhs(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(b), CH_B)
    g.fill(0.0, CH_X)
    its_g, _, _, _ = g.batch_mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=60, use_graph=True)
    xg = g.payload(CH_X)
    g.fill(0.0, CH_X)
    its_e, _, _, _ = g.batch_mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=60, use_graph=False)
    xe = g.payload(CH_X)
    assert np.array_equal(its_g, its_e)
    assert np.array_equal(xg, xe)


def test_unassigned_block_is_an_error(gpulib):
    G = gpulib
    levels, vol = _layout()
    vol = vol.copy()
    vol[np.nonzero(levels == 0)[0][0]] = -1
    g = G.MultiresSparseGrid(RES, RES, RES, BS, 2, G.F32)
    try:
        g.set_levels(levels)
        g.setRefinementMap(0.0)
        with pytest.raises(G.MsbgGpuError) as e:
            g.batch_set_volumes(vol, 8)
        assert e.value.code == G.ERR_ARG
    finally:
        g.close()
