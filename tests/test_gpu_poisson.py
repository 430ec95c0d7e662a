"""GPU sparse Poisson pieces against the FP64 CPU restatement (oracle/msbg_oracle.c).

The reference release has no Poisson driver and no test for these kernels, so
parity is against the restatement of its formulas (src/msbg3.cpp:1281-1296,
src/msbg.cpp:4524-4872): operator, smoother, V-cycle and dot/AXPBY within
FP32 tolerances; the full MG-PCG solve reaches the FP64-checked tolerance and
matches the FP64 solution.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2
from msbg_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CH_X, CH_B, CH_Y, CH_CX, CH_CY, CH_CZ, CH_D, CH_Q = range(1, 9)


def _layout(G, P, res=128, bs=16, n_spheres=6, seed_idx=1):
    pts = W.sphere_cloud(res, n_spheres, 3000, seed=W.workload_seed(3, seed_idx))
    g = G.MultiresSparseGrid(res, res, res, bs, 3, G.F32)
    d = g.to_device(pts)
    g.mark_points(d, len(pts), 4.0)
    g.levels_from_marks()
    g.regularizeRefinementMap()
    g.setRefinementMap(0.0)
    d.free()
    for ch in (CH_X, CH_B, CH_Y, CH_CX, CH_CY, CH_CZ, CH_D, CH_Q):
        g.channel_create(ch, G.F32)
    bids = g.active_blocks().astype(np.int64)
    prob = P.PoissonProblem(bids, (g.nbx, g.nby, g.nbz), bs, seed=4242)
    g.poisson_procedural_coefficients(4242, CH_CX, CH_CY, CH_CZ, CH_D)
    return g, prob


def _rand(prob, rng):
    return np.where(prob.act > 0, rng.standard_normal(prob.act.shape), 0.0)


@pytest.fixture(scope="module", params=[(128, 16), (256, 32), (64, 8)], ids=["bs16", "bs32", "bs8"])
def setup(request, gpulib, port):
    res, bs = request.param
    g, prob = _layout(gpulib, port, res=res, bs=bs)
    yield gpulib, port, g, prob
    g.close()


def test_coefficients_bit_identical(setup):
    G, P, g, prob = setup
    for ch, ref in ((CH_CX, prob.cx), (CH_CY, prob.cy), (CH_CZ, prob.cz), (CH_D, prob.d)):
        got = prob.dense(g.payload(ch))
        assert np.array_equal(got.astype(np.float32), ref.astype(np.float32))


def test_multiply_and_residual(setup):
    G, P, g, prob = setup
    rng = np.random.default_rng(1)
    x, b = _rand(prob, rng).astype(np.float32), _rand(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(x), CH_X)
    g.upload_payload(prob.payload(b), CH_B)
    g.multiplyLaplacianMatrix(CH_X, CH_B, CH_Y, calcResidual=False)
    assert rel_l2(prob.dense(g.payload(CH_Y)), prob.apply(x)) < 1e-6
    g.multiplyLaplacianMatrix(CH_X, CH_B, CH_Y, calcResidual=True)
    assert rel_l2(prob.dense(g.payload(CH_Y)), prob.apply(x, b)) < 1e-6


@pytest.mark.parametrize("reverse", [False, True])
def test_relax_tiles(setup, reverse):
    """relax = tile-coloured smoothing passes (16^3 / 8^3 tiles, in-tile red-black)."""
    G, P, g, prob = setup
    rng = np.random.default_rng(2)
    x, b = _rand(prob, rng).astype(np.float32), _rand(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(x), CH_X)
    g.upload_payload(prob.payload(b), CH_B)
    g.relax_tiles(CH_X, CH_B, 2, reverseOrder=reverse)
    want = prob.smooth(x, b, 2, reverse=reverse)
    assert rel_l2(prob.dense(g.payload(CH_X)), want) < 1e-5


@pytest.mark.parametrize("pre,post,k,coarsest", [(1, 1, 3, 0), (2, 1, 2, 200)])
def test_vcycle_params_match_fp64(setup, pre, post, k, coarsest):
    """Other pass / in-tile sweep counts and the red-black coarsest solver give the
    restatement's V-cycle too."""
    G, P, g, prob = setup
    p2 = P.PoissonProblem(prob.bids, prob.nb, prob.bs, seed=4242, pre=pre, post=post, tile_iters=k,
                          coarsest_iter=coarsest)
    rng = np.random.default_rng(8)
    b = _rand(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(b), CH_B)
    g.poisson_set_params(pre, post, k, coarsest)
    try:
        g.vcycle(CH_X, CH_B)
    finally:
        g.poisson_set_params()
    want, _ = p2.vcycle(b)
    assert rel_l2(prob.dense(g.payload(CH_X)), want) < 1e-5


def test_vcycle_matches_fp64(setup):
    G, P, g, prob = setup
    rng = np.random.default_rng(3)
    b = _rand(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(b), CH_B)
    g.vcycle(CH_X, CH_B)
    want, nlev = prob.vcycle(b)
    assert len(g.mg_info()) == nlev
    assert rel_l2(prob.dense(g.payload(CH_X)), want) < 1e-5


def test_dot_and_axpby(setup):
    G, P, g, prob = setup
    rng = np.random.default_rng(4)
    x, y, q = (_rand(prob, rng).astype(np.float32) for _ in range(3))
    px, py, pq = prob.payload(x), prob.payload(y), prob.payload(q)
    g.upload_payload(px, CH_X)
    g.upload_payload(py, CH_Y)
    g.upload_payload(pq, CH_Q)
    want = float(np.dot(px.astype(np.float64).ravel(), py.astype(np.float64).ravel()))
    assert abs(g.dotProdChannel(CH_X, CH_Y) - want) <= 1e-9 * abs(want) + 1e-9
    g.AXPBYChannel(0.5, CH_X, -2.0, CH_Y)
    assert rel_l2(g.payload(CH_Y), 0.5 * px.astype(np.float64) - 2.0 * py) < 1e-6
    g.upload_payload(py, CH_Y)
    g.AXPBYChannelCombined(0.25, 1.5, CH_Q, CH_X, CH_Y)  # X += aP ; P = Q + bP  with P = CH_Y
    assert rel_l2(g.payload(CH_X), px.astype(np.float64) + 0.25 * py) < 1e-6
    assert rel_l2(g.payload(CH_Y), pq.astype(np.float64) + 1.5 * py) < 1e-6


def test_dot_nonfinite_is_an_error(setup):
    G, P, g, prob = setup
    x = np.zeros((len(prob.bids), prob.bs ** 3), np.float32)
    x[0, 5] = np.inf
    g.upload_payload(x, CH_X)
    with pytest.raises(G.MsbgGpuError) as e:
        g.dotProdChannel(CH_X, CH_X)
    assert e.value.code == G.ERR_NONFINITE


def test_mgpcg_solve_to_tolerance(setup):
    G, P, g, prob = setup
    rng = np.random.default_rng(5)
    b = _rand(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(b), CH_B)
    g.fill(0.0, CH_X)
    it, rel = g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=100)
    x = prob.dense(g.payload(CH_X))
    check = prob.rel_residual(x, b)          # FP64 check on the CPU
    assert rel <= 1e-6 and check <= 1.5e-6, (it, rel, check)
    xs, it_ref, rel_ref = prob.solve(b.astype(np.float64), 1e-6)
    assert abs(it - it_ref) <= 2
    assert rel_l2(x, xs) < 1e-5


def test_mixed_precision_solve_to_tolerance(setup):
    """FP16-storage inner MG-PCG inside FP32 iterative refinement reaches the same
    FP64-checked tolerance and the same solution as the FP32 solve."""
    G, P, g, prob = setup
    rng = np.random.default_rng(6)
    b = _rand(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(b), CH_B)
    g.fill(0.0, CH_X)
    outer, inner, rel = g.mgpcg_solve_mixed(CH_X, CH_B, tol=1e-6, max_outer=12, inner_tol=1e-2, max_inner=40)
    x = prob.dense(g.payload(CH_X))
    check = prob.rel_residual(x, b)
    assert rel <= 1e-6 and check <= 1.5e-6, (outer, inner, rel, check)
    assert 1 <= outer <= 12
    xs, _, _ = prob.solve(b.astype(np.float64), 1e-6)
    assert rel_l2(x, xs) < 1e-5


def test_mixed_precision_warm_start_and_zero_rhs(setup):
    G, P, g, prob = setup
    g.fill(0.0, CH_B)
    g.fill(0.0, CH_X)
    outer, inner, rel = g.mgpcg_solve_mixed(CH_X, CH_B, tol=1e-6)
    assert outer == 0 and inner == 0 and rel == 0.0
    assert not np.any(g.payload(CH_X))
    # an exact start needs no outer step
    rng = np.random.default_rng(7)
    b = _rand(prob, rng).astype(np.float32)
    g.upload_payload(prob.payload(b), CH_B)
    g.fill(0.0, CH_X)
    g.mgpcg_solve(CH_X, CH_B, tol=5e-7, max_iter=100)
    outer, inner, rel = g.mgpcg_solve_mixed(CH_X, CH_B, tol=1e-6)
    assert outer == 0 and inner == 0 and rel <= 1e-6


def test_nonfinite_rhs_is_reported_not_solved(setup):
    """A NaN entering from the host (here in B, and then in the start X) ends both solves with
    MSBG_GPU_ERR_DIVERGED instead of a result; the context keeps working afterwards."""
    G, P, g, prob = setup
    rng = np.random.default_rng(9)
    b = _rand(prob, rng).astype(np.float32)
    pb = prob.payload(b)
    bad = pb.copy()
    bad[len(bad) // 2, 17] = np.nan
    g.upload_payload(bad, CH_B)
    g.fill(0.0, CH_X)
    for solve in (lambda: g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=50),
                  lambda: g.mgpcg_solve_mixed(CH_X, CH_B, tol=1e-6)):
        with pytest.raises(G.MsbgGpuError) as e:
            solve()
        assert e.value.code == G.ERR_DIVERGED
    g.upload_payload(pb, CH_B)
    x0 = np.zeros_like(pb)
    x0[0, 3] = np.inf
    g.upload_payload(x0, CH_X)
    with pytest.raises(G.MsbgGpuError) as e:
        g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=50)
    assert e.value.code == G.ERR_DIVERGED
    g.fill(0.0, CH_X)
    it, rel = g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=100)
    assert rel <= 1e-6 and it > 0


def test_non_spd_coefficients_diverge(gpulib, port):
    """A host-built coefficient set whose diagonal is the negated sum of the face
    coefficients (a negative definite operator) is refused with MSBG_GPU_ERR_DIVERGED, at the
    latest by the solve; nothing faults."""
    G, P = gpulib, port
    g, prob = _layout(G, P, res=64, bs=8)
    try:
        d = g.payload(CH_D)
        g.upload_payload(-d, CH_D)
        with pytest.raises(G.MsbgGpuError) as e:
            g.poisson_set_coefficients(CH_CX, CH_CY, CH_CZ, CH_D)
            rng = np.random.default_rng(10)
            g.upload_payload(prob.payload(_rand(prob, rng).astype(np.float32)), CH_B)
            g.fill(0.0, CH_X)
            g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=200)
        assert e.value.code == G.ERR_DIVERGED
        # a valid set on the same context solves again
        g.upload_payload(d, CH_D)
        g.poisson_set_coefficients(CH_CX, CH_CY, CH_CZ, CH_D)
        rng = np.random.default_rng(11)
        g.upload_payload(prob.payload(_rand(prob, rng).astype(np.float32)), CH_B)
        g.fill(0.0, CH_X)
        it, rel = g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=100)
        assert rel <= 1e-6
    finally:
        g.close()


def test_launch_shape_autotuner(gpulib):
    """The operator's launch-shape autotuner on a layout large enough to tune (a 256^3
    block of bs 32, 16.7 M cells): it picks one valid shape per (level, precision, mode)
    it met, and the solve reaches the tolerance in the same iterations and to the same
    solution (FP32) as with the static shapes."""
    G = gpulib
    g = G.MultiresSparseGrid(256, 256, 256, 32, 2, G.F32)
    try:
        g.set_levels(np.zeros(8 ** 3, np.int32))
        g.setRefinementMap(0.0)
        for ch in (CH_X, CH_B, CH_CX, CH_CY, CH_CZ, CH_D):
            g.channel_create(ch, G.F32)
        g.poisson_procedural_coefficients(4242, CH_CX, CH_CY, CH_CZ, CH_D)
        rng = np.random.default_rng(11)
        b = rng.standard_normal((8 ** 3, 32 ** 3)).astype(np.float32)
        b -= b.mean()
        g.upload_payload(b, CH_B)
        g.poisson_tuning(0)
        g.fill(0.0, CH_X)
        it0, rel0 = g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=100)
        x0 = g.payload(CH_X)
        assert g.poisson_tuning() == []
        g.poisson_tuning(1)
        g.fill(0.0, CH_X)
        it1, rel1 = g.mgpcg_solve(CH_X, CH_B, tol=1e-6, max_iter=100)
        x1 = g.payload(CH_X)
        shapes = g.poisson_tuning()
        assert shapes, "a 16.7 M-cell level is tuned"
        keys = [s[:3] for s in shapes]
        assert len(keys) == len(set(keys))
        for level, nbytes, mode, cpt, grid in shapes:
            assert nbytes == 4 and cpt in (4, 8) and grid in (608, 1216, 2432)
            assert mode in (0, 1, 2) and (mode != 2 or cpt == 4)
        assert rel0 <= 1e-6 and rel1 <= 1e-6 and it0 == it1
        assert rel_l2(x1, x0) < 1e-5
    finally:
        g.close()


@pytest.mark.parametrize("reverse", [False, True])
def test_relax_tiles_fp16_storage(setup, reverse):
    """The mixed solve's FP16-storage tile smoother (FP16 x, b and coefficients, FP32
    arithmetic) against the FP64 restatement on the same inputs: within the FP16
    rounding of the stored values (unit roundoff 4.9e-4)."""
    G, P, g, prob = setup
    rng = np.random.default_rng(12)
    x = _rand(prob, rng).astype(np.float16).astype(np.float64)
    b = _rand(prob, rng).astype(np.float16).astype(np.float64)
    chx, chb = 10, 11
    g.channel_create(chx, G.F16)
    g.channel_create(chb, G.F16)
    g.upload_payload(prob.payload(x).astype(np.float16), chx)
    g.upload_payload(prob.payload(b).astype(np.float16), chb)
    g.relax_tiles(chx, chb, 2, reverseOrder=reverse)
    got = prob.dense(g.payload(chx).astype(np.float64))
    want = prob.smooth(x, b, 2, reverse=reverse)
    assert rel_l2(got, want) < 2e-3
