"""The CPU restatement against fixtures made by the reference itself (tests/golden/make_golden.py):

* the solver building blocks (reference_solver.npz): multiplyLaplacianMatrixOpt (Y = A X, its
  dot product sum(Y X), and B - A X), dotProdChannel, AXPBYChannelCombined and the block
  smoother relax() / relaxBlockList on seeded layouts with block edges 16 and 8.  The
  reference's operator is (1/D) X - sum W X_nb with 1/diagonal stored in CH_DIAGONAL, so it
  differs from the restatement's d X - sum c X_nb (FP64) by the rounding of 1/(1/d) and of
  FP32: the tolerance is rel-L2 1e-6 (measured about 5e-8).  The block smoother, which reads
  1/diagonal as the reference does, follows the reference's compiled arithmetic and matches it
  bit for bit;
* downsampleFloatChannelNew to multigrid level 1 on seeded 3-level channels
  (reference_downsample.npz): bit for bit;
* the 512^3 surface workload at full size (reference_surface512.npz): active set, levels,
  flags and particle counts bit for bit, the FP32 fields' per-block sums and voxel sample within
  rel-L2 1e-5 (the reference builds with -ffast-math; its own tolerance is 1e-5,
  src/msbg.h:3328), the uint16 sample within 8 quanta.
Where the reference is built here (x86-64), fresh reference runs on other seeds are checked too.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2

import halo_cases as H
import solver_cases as S

GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def solver_gold():
    return dict(np.load(os.path.join(GOLD, "reference_solver.npz")))


@pytest.mark.parametrize("case", S.SOLVER_CASES, ids=[c[0] for c in S.SOLVER_CASES])
def test_operator_dot_axpby_match_reference(port, solver_gold, case):
    name, res, bs, nblk, seed = case
    bids, nb, prob, (x, b, q, p) = S.solver_case(port, res, bs, nblk, seed)
    ax = prob.payload(prob.apply(prob.dense(x))).astype(np.float64)
    assert rel_l2(solver_gold[f"{name}_ax"], ax) < 1e-6
    assert rel_l2(solver_gold[f"{name}_residual"], b.astype(np.float64) - ax) < 1e-6
    dots = solver_gold[f"{name}_dots"]
    assert abs(dots[0] - float((ax * x).sum())) <= 1e-6 * abs(dots[0])
    assert abs(dots[1] - float((x.astype(np.float64) * b).sum())) <= 1e-9 * abs(dots[1])
    assert rel_l2(solver_gold[f"{name}_axpby_x"], x + S.AXPBY_A * p.astype(np.float64)) < 1e-7
    assert rel_l2(solver_gold[f"{name}_axpby_p"], q + S.AXPBY_B * p.astype(np.float64)) < 1e-7


@pytest.mark.parametrize("case", S.SOLVER_CASES, ids=[c[0] for c in S.SOLVER_CASES])
@pytest.mark.parametrize("passes,reverse", S.RELAX_RUNS)
def test_block_smoother_matches_reference(port, solver_gold, case, passes, reverse):
    name, res, bs, nblk, seed = case
    bids, nb, prob, (x, b, q, p) = S.solver_case(port, res, bs, nblk, seed)
    got = prob.payload(prob.relax_reference(prob.dense(x), prob.dense(b), passes=passes, reverse=reverse))
    want = solver_gold[f"{name}_relaxed_{passes}_{int(reverse)}"]
    assert np.array_equal(np.asarray(got, np.float32).view(np.uint32), want.view(np.uint32))
    assert rel_l2(want, x) > 0.1  # the smoother did move the field


def test_downsample_matches_reference_bit_for_bit(port):
    gold = dict(np.load(os.path.join(GOLD, "reference_downsample.npz")))
    for nb, bsx, seed in H.DOWNSAMPLE_CASES:
        lv, st, pay = H.halo_case(nb, bsx, 3, seed, "f32", lambda *a: port.regularize(*a)[0])
        key = "x".join(map(str, nb)) + f"_bs{bsx}"
        g = port.grid(*(n * bsx for n in nb), bsx, port.F32)
        bids = gold[f"{key}_bids"]
        assert np.array_equal(bids, np.nonzero(lv == 0)[0])
        for mode, simple in (("gauss", False), ("mean", True)):
            got, skipped = port.restrict_level(g, lv, st, pay, 0, bids, simple, H.DOWNSAMPLE_EMPTY, H.DOWNSAMPLE_FULL)
            assert skipped == 0
            assert np.array_equal(got.view(np.uint32), gold[f"{key}_{mode}"].view(np.uint32)), (key, mode)


def test_surface512_full_size_matches_reference(port):
    from msbg_gb300 import workloads as W
    gold = dict(np.load(os.path.join(GOLD, "reference_surface512.npz")))
    spec = W.SURFACE_512
    pts = W.make_points(spec, 1)
    idx = gold["sample_index"]
    for name, storage in (("f32", port.F32), ("u16", port.U16)):
        p = port.surface_pipeline(pts, spec["res"], spec["bsx"], storage=storage, n_iter=spec["n_iter"],
                                  dt=spec["dt"])
        assert np.array_equal(p.active_bids, gold["active_bids"])
        assert np.array_equal(p.levels, gold["levels"]) and np.array_equal(p.flags, gold["flags"])
        assert p.n_act_particles == int(gold["n_act_particles"])
        for stage, field in (("final", p.after_finalize), ("pde", p.after_pde)):
            if name == "f32":
                assert rel_l2(field.astype(np.float64).sum(1), gold[f"f32_{stage}_block_sums"]) < 1e-5
                assert rel_l2(field.reshape(-1)[idx], gold[f"f32_{stage}_sample"]) < 1e-5
            else:
                d = np.abs(field.reshape(-1)[idx].astype(np.int64) - gold[f"u16_{stage}_sample"].astype(np.int64))
                assert d.max() <= 8
    assert len(gold["active_bids"]) > 3000


def _ref():
    import oracle_io as O
    if not O.ref_available():
        pytest.skip("the reference is not built on this host")
    return O


def test_fresh_reference_solver_and_smoother(port):
    O = _ref()
    bids, nb, prob, (x, b, q, p) = S.solver_case(port, 64, 16, 12, 20261203 + 955)
    coef = [prob.payload(v).astype(np.float32) for v in (prob.cx, prob.cy, prob.cz, prob.d)]
    r = O.run_reference_solver(64, 64, 64, 16, bids, x, b, q, p, *coef, relax_passes=2, reverse=False)
    ax = prob.payload(prob.apply(prob.dense(x)))
    assert rel_l2(r["ax"], ax) < 1e-6
    got = prob.payload(prob.relax_reference(prob.dense(x), prob.dense(b), passes=2, reverse=False))
    assert np.array_equal(np.asarray(got, np.float32).view(np.uint32), r["relaxed"].view(np.uint32))


def test_fresh_reference_downsample(port):
    """Bit for bit on the fixtures' kind of data (payloads in multiples of 2^-16, constant
    blocks 0.25 / 0.75, so every weighted product is exact).  With values whose products
    round (constant blocks 0.1 / 0.9), the reference's -ffast-math build reassociates the
    4x4x4 sum in ways no single order reproduces; the results then differ in the last bit
    of a few values in a thousand."""
    O = _ref()
    lv, st, pay = H.halo_case((5, 4, 3), 16, 3, 20261203 + 965, "f32", lambda *a: port.regularize(*a)[0])
    g = port.grid(80, 64, 48, 16, port.F32)
    bids, vals = O.run_reference_downsample(80, 64, 48, 16, 3, lv, st, pay, False, 0.25, 0.75)
    got, _ = port.restrict_level(g, lv, st, pay, 0, bids, False, 0.25, 0.75)
    assert np.array_equal(got.view(np.uint32), vals.view(np.uint32))
    bids, vals = O.run_reference_downsample(80, 64, 48, 16, 3, lv, st, pay, False, 0.1, 0.9)
    got, _ = port.restrict_level(g, lv, st, pay, 0, bids, False, 0.1, 0.9)
    ulp = np.abs(got.view(np.int32).astype(np.int64) - vals.view(np.int32).astype(np.int64))
    assert ulp.max() <= 1 and (ulp > 0).mean() < 0.005


# ------------------------------------------- the solver operator on multi-resolution layouts

def _multires_key(nb, bsx):
    return "x".join(map(str, nb)) + f"_bs{bsx}"


@pytest.mark.parametrize("case", H.MULTIRES_CASES, ids=[_multires_key(c[0], c[1]) for c in H.MULTIRES_CASES])
def test_multires_operator_matches_reference(port, case):
    """multiplyLaplacianMatrixOpt on a 3-level layout, blocks of neighbouring levels meeting
    through procNeighMixedRes2 (src/msbg3.cpp:46-161): the restatement equals the reference
    bit for bit (Y = A X and B - A X), the FP64 dot product to rounding."""
    gold = dict(np.load(os.path.join(GOLD, "reference_multires.npz")))
    nb, bsx, seed = case
    key = _multires_key(nb, bsx)
    lv, x, b, dinv = H.multires_case(nb, bsx, 3, seed, lambda *a: port.regularize(*a)[0])
    assert np.array_equal(lv, gold[f"{key}_levels"])
    assert len(np.unique(lv)) == 3  # every level present, so both kinds of mixed faces occur
    dot, y, r = port.multiply_laplacian_levels(*(n * bsx for n in nb), bsx, 3, lv, x, b, dinv)
    assert np.array_equal(y.view(np.uint32), gold[f"{key}_y"].view(np.uint32))
    assert np.array_equal(r.view(np.uint32), gold[f"{key}_r"].view(np.uint32))
    assert abs(dot - float(gold[f"{key}_dot"])) <= 1e-12 * abs(dot)


@pytest.mark.parametrize("case", H.MULTIRES_CASES, ids=[_multires_key(c[0], c[1]) for c in H.MULTIRES_CASES])
def test_multires_block_smoother_matches_reference(port, case):
    """relaxBlockList on a 3-level layout (the operator's halo with mixed-resolution faces,
    5 block-local iterations, omega 6/7): the restatement equals the reference bit for bit,
    one forward pass and two passes in the reverse order."""
    gold = dict(np.load(os.path.join(GOLD, "reference_multires.npz")))
    nb, bsx, seed = case
    key = _multires_key(nb, bsx)
    lv, x, b, dinv = H.multires_case(nb, bsx, 3, seed, lambda *a: port.regularize(*a)[0])
    for passes, rev in H.MULTIRES_RELAX_RUNS:
        got = port.relax_levels(*(n * bsx for n in nb), bsx, 3, lv, x, b, dinv, passes=passes, reverse=rev)
        want = gold[f"{key}_relaxed_{passes}_{int(rev)}"]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (passes, rev)
        assert rel_l2(want, x) > 0.1  # the smoother did move the field


def test_multires_faces_weigh_the_other_level(port):
    """Known answers of the mixed-resolution faces: X = 1 everywhere and the diagonal channel
    1/6 make Y = 6 h - S vanish inside a level and leave, on a fine cell next to a coarser
    block, h (1 - 2/3) from the one face (the coarse side weighs 2/3), and on a coarse cell
    next to a finer block h (1 - 4/3) (four fine cells of 1/3)."""
    nb, bsx = (2, 1, 1), 8
    lv = np.array([0, 1], np.int32)
    n0, n1 = bsx ** 3, (bsx // 2) ** 3
    x = np.ones(n0 + n1, np.float32)
    dinv = np.full(n0 + n1, np.float32(1) / np.float32(6), np.float32)
    dot, y, r = port.multiply_laplacian_levels(2 * bsx, bsx, bsx, bsx, 2, lv, x, x, dinv)
    y0 = y[:n0].reshape(bsx, bsx, bsx)
    y1 = y[n0:].reshape(bsx // 2, bsx // 2, bsx // 2)
    # interior cells of either block: 6 h X / 6 ... minus the six neighbours h X
    assert abs(float(y0[3, 3, 3])) < 1e-6 and abs(float(y1[1, 1, 1])) < 1e-6
    # level-0 cell at x = bsx-1 (face to the coarser block): 1 - 2/3
    assert abs(float(y0[3, 3, bsx - 1]) - (1 - 2 / 3)) < 1e-6
    # level-1 cell at x = 0 (face to the finer block), h = 2: 2 (1 - 4/3)
    assert abs(float(y1[1, 1, 0]) - 2 * (1 - 4 / 3)) < 1e-5


def test_multires_restatement_matches_fresh_reference(port):
    O = _ref()
    nb, bsx = (4, 3, 5), 8
    lv, x, b, dinv = H.multires_case(nb, bsx, 3, 20261203 + 995, lambda *a: port.regularize(*a)[0])
    ref = O.run_reference_multires(*(n * bsx for n in nb), bsx, 3, lv, x, b, dinv)
    dot, y, r = port.multiply_laplacian_levels(*(n * bsx for n in nb), bsx, 3, lv, x, b, dinv)
    assert np.array_equal(y.view(np.uint32), ref["y"].view(np.uint32))
    assert np.array_equal(r.view(np.uint32), ref["r"].view(np.uint32))
    assert abs(dot - ref["dot"]) <= 1e-12 * abs(dot)


# ------------------------------------------------- the solver operator at a dense multigrid level

@pytest.mark.parametrize("case", H.DENSE_CASES, ids=[f"{c[0]}x{c[1]}x{c[2]}_L{c[4]}" for c in H.DENSE_CASES])
def test_dense_level_operator_matches_reference(port, case):
    """multiplyLaplacianMatrixOpt at the first dense multigrid level (the masked 7-point
    operator with face areas, src/msbg3.cpp:166-403): the restatement equals the reference bit
    for bit, Y = A X and B - A X, skipped groups and zero diagonals included."""
    gold = dict(np.load(os.path.join(GOLD, "reference_dense.npz")))
    sx0, sy0, sz0, bsx, nl, seed = case
    key = f"{sx0}x{sy0}x{sz0}_L{nl}"
    flags, x, b, dinv, ax, ay, az = H.dense_case(sx0, sy0, sz0, nl, seed)
    y, r = port.multiply_laplacian_dense(flags, x, b, dinv, ax, ay, az, 2 ** nl)
    assert np.array_equal(y.view(np.uint32), gold[f"{key}_y"].view(np.uint32))
    assert np.array_equal(r.view(np.uint32), gold[f"{key}_r"].view(np.uint32))
    assert np.isinf(y).any() and (y == 0).mean() > 0.1  # zero diagonals and non-fluid cells occur


@pytest.mark.parametrize("case", H.DENSE_CASES, ids=[f"{c[0]}x{c[1]}x{c[2]}_L{c[4]}" for c in H.DENSE_CASES])
def test_dense_level_smoother_matches_reference(port, case):
    """relax() at the first dense multigrid level (omega-Jacobi between X and a temporary
    channel): the restatement equals the reference bit for bit after an odd and an even count."""
    gold = dict(np.load(os.path.join(GOLD, "reference_dense.npz")))
    sx0, sy0, sz0, bsx, nl, seed = case
    key = f"{sx0}x{sy0}x{sz0}_L{nl}"
    flags, x, b, dinv, ax, ay, az = H.dense_case(sx0, sy0, sz0, nl, seed)
    for it in H.DENSE_RELAX_ITERS:
        got = port.relax_dense(flags, x, b, dinv, ax, ay, az, 2 ** nl, it)
        assert np.array_equal(got.view(np.uint32), gold[f"{key}_relaxed_{it}"].view(np.uint32)), it
