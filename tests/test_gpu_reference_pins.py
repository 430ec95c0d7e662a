"""The GPU against fixtures made by the reference itself, and the block-list forms of the
reference's calls.

* Solver building blocks (reference_solver.npz): msbg_gpu_multiply_laplacian (Y = A X and its
  dot sum(Y X), B - A X), msbg_gpu_dot, msbg_gpu_axpby_combined and msbg_gpu_relax (the
  reference's block smoother) against multiplyLaplacianMatrixOpt, dotProdChannel,
  AXPBYChannelCombined and relax() run by the reference: the operator, its residual, AXPBY and
  the smoother bit for bit (the operator and the smoother follow the reference's compiled
  arithmetic, with its 1/diagonal formed from the diagonal), dots within 1e-6 relative (FP64
  sums in another order).  The smoother also equals the CPU restatement bit for bit.
* Block lists: a listed call touches only the listed value blocks, and equals the whole-layout
  call there; sweeps with a list equal the restatement's sweeps of that list bit for bit.
* downsampleFloatChannelNew on multi-level channels (reference_downsample.npz): bit for bit.
* multiplyLaplacianMatrixOpt on 3-level layouts with mixed-resolution faces
  (reference_multires.npz, msbg_gpu_multiply_laplacian_levels): Y = A X and B - A X bit for
  bit, the dot product to FP64 rounding.
* The 512^3 surface workload at full size (reference_surface512.npz): active set, levels,
  flags and particle counts bit for bit; FP32 field sums and voxel sample within rel-L2 1e-5
  for the EXACT and FAST sweep variants; the uint16 sample within 8 quanta.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2
from msbg_gb300 import workloads as W

import halo_cases as H
import solver_cases as S

pytestmark = pytest.mark.gpu
GOLD = os.path.join(ROOT, "tests", "golden")
CH_X, CH_B, CH_Q, CH_P, CH_Y, CH_CX, CH_CY, CH_CZ, CH_D = range(1, 10)


@pytest.fixture(scope="module")
def solver_gold():
    return dict(np.load(os.path.join(GOLD, "reference_solver.npz")))


def _solver_grid(G, res, bs, bids):
    nb3 = (res // bs) ** 3
    g = G.MultiresSparseGrid(res, res, res, bs, 3, G.F32)
    lv = np.full(nb3, 2, np.int32)
    lv[bids] = 0
    g.set_levels(lv)
    g.setRefinementMap(0.0)
    for c in range(CH_X, CH_D + 1):
        g.channel_create(c, G.F32)
    g.poisson_procedural_coefficients(S.COEFF_SEED, CH_CX, CH_CY, CH_CZ, CH_D)
    assert np.array_equal(g.active_blocks(), bids)
    return g


@pytest.mark.parametrize("case", S.SOLVER_CASES, ids=[c[0] for c in S.SOLVER_CASES])
def test_solver_blocks_match_reference(gpulib, port, solver_gold, case):
    G = gpulib
    name, res, bs, nblk, seed = case
    bids, nb, prob, (x, b, q, p) = S.solver_case(port, res, bs, nblk, seed)
    g = _solver_grid(G, res, bs, bids)
    try:
        g.upload_payload(x, CH_X)
        g.upload_payload(b, CH_B)
        dyx = g.multiplyLaplacianMatrixOpt(0, 0, CH_X, CH_B, 0.0, CH_Y, withDotprod=True)
        assert np.array_equal(g.payload(CH_Y).view(np.uint32), solver_gold[f"{name}_ax"].view(np.uint32))
        dots = solver_gold[f"{name}_dots"]
        assert abs(dyx - dots[0]) <= 1e-6 * abs(dots[0])
        g.multiplyLaplacianMatrixOpt(G.OPT_CALC_RESIDUAL, 0, CH_X, CH_B, 0.0, CH_Y)
        assert np.array_equal(g.payload(CH_Y).view(np.uint32), solver_gold[f"{name}_residual"].view(np.uint32))
        assert abs(g.dotProdChannel(CH_X, CH_B) - dots[1]) <= 1e-9 * abs(dots[1])
        g.upload_payload(q, CH_Q)
        g.upload_payload(p, CH_P)
        g.AXPBYChannelCombined(S.AXPBY_A, S.AXPBY_B, CH_Q, CH_X, CH_P)
        assert np.array_equal(g.payload(CH_X).view(np.uint32), solver_gold[f"{name}_axpby_x"].view(np.uint32))
        assert np.array_equal(g.payload(CH_P).view(np.uint32), solver_gold[f"{name}_axpby_p"].view(np.uint32))
        for passes, rev in S.RELAX_RUNS:
            g.upload_payload(x, CH_X)
            g.relax(0, int(rev), 0, CH_X, CH_B, G.CH_NULL, passes)
            got = g.payload(CH_X)
            assert np.array_equal(got.view(np.uint32), solver_gold[f"{name}_relaxed_{passes}_{int(rev)}"].view(np.uint32))
            want = prob.payload(prob.relax_reference(prob.dense(x), prob.dense(b), passes=passes, reverse=rev))
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (passes, rev)
    finally:
        g.close()


def test_block_lists_touch_only_listed_blocks(gpulib, port):
    G = gpulib
    name, res, bs, nblk, seed = S.SOLVER_CASES[0]
    bids, nb, prob, (x, b, q, p) = S.solver_case(port, res, bs, nblk, seed)
    g = _solver_grid(G, res, bs, bids)
    try:
        pick = np.array([0, 3, 5], np.int64)
        sub = bids[pick]
        listed = np.isin(bids, sub)
        g.upload_payload(x, CH_X)
        g.upload_payload(b, CH_B)
        g.multiplyLaplacianMatrix(CH_X, CH_B, CH_Y)
        full = g.payload(CH_Y)
        sentinel = np.full_like(x, 7.0)
        g.upload_payload(sentinel, CH_Y)
        dyx = g.multiplyLaplacianMatrixOpt(0, 0, CH_X, CH_B, 0.0, CH_Y, withDotprod=True, blockList=sub)
        y = g.payload(CH_Y)
        assert np.array_equal(y[~listed], sentinel[~listed])
        assert rel_l2(y[listed], full[listed]) < 1e-6
        assert abs(dyx - float((y[listed].astype(np.float64) * x[listed]).sum())) <= 1e-9 * abs(dyx) + 1e-12
        # a listed block without payload is skipped; an id outside the grid is an error
        nb3 = (res // bs) ** 3
        empty_bid = int(np.setdiff1d(np.arange(nb3), bids)[0])
        d_xb = g.dotProdChannel(CH_X, CH_B, 0, np.append(sub, empty_bid))
        assert abs(d_xb - float((x[listed].astype(np.float64) * b[listed]).sum())) <= 1e-9 * abs(d_xb)
        with pytest.raises(G.MsbgGpuError) as e:
            g.dotProdChannel(CH_X, CH_B, 0, np.array([nb3 + 5], np.int32))
        assert e.value.code == G.ERR_ARG
        g.upload_payload(q, CH_Q)
        g.upload_payload(p, CH_P)
        g.AXPBYChannel(0.5, CH_Q, 2.0, CH_P, 9999, 0, sub)
        pp = g.payload(CH_P)
        assert np.array_equal(pp[~listed], p[~listed])
        assert rel_l2(pp[listed], 0.5 * q[listed].astype(np.float64) + 2.0 * p[listed]) < 1e-7
        # the block smoother on a sub-list equals the restatement's on that list
        g.relax(0, 0, 0, CH_X, CH_B, G.CH_NULL, 1, blockList=sub)
        want = prob.payload(prob.relax_reference(prob.dense(x), prob.dense(b), passes=1, block_list=sub))
        assert np.array_equal(g.payload(CH_X).view(np.uint32), want.view(np.uint32))
    finally:
        g.close()


@pytest.mark.parametrize("storage", ["f32", "u16"])
@pytest.mark.parametrize("lapl", ["mcf8", "jacobi_rb", "jacobi_pp"])
def test_sweeps_with_a_block_list_match_restatement(gpulib, port, golden, storage, lapl):
    """applyChannelPdeFast with a block list (the demo passes &activeBlocks): here every third
    value block of the golden layout; the EXACT variant equals the restatement sweeping the
    same list bit for bit, and unlisted blocks keep their values."""
    G, P = gpulib, port
    lt = {"mcf8": -(4 + G.OPT_8_COLOR_SCHEME), "jacobi_rb": -17, "jacobi_pp": 17}[lapl]
    st = {"f32": (G.F32, P.F32), "u16": (G.U16, P.U16)}[storage]
    pts, res, bsx = golden["points"], int(golden["res"]), int(golden["bsx"])
    r = G.surface_pipeline(pts, res, bsx, storage=st[0], n_iter=0)
    bids = r["active_bids"]
    sub = bids[::3]
    init = r["after_finalize"]
    g = G.MultiresSparseGrid(res, res, res, bsx, 3, st[0])
    try:
        nb3 = (res // bsx) ** 3
        lv = np.full(nb3, 2, np.int32)
        lv[bids] = 0
        g.set_levels(lv)
        g.setRefinementMap(0.0)
        g.upload_payload(init, 0)
        g.applyChannelPdeFast(0, blockList=sub, laplTyp=lt, doConstrZeroOne=1, numIter=3, timeStep=0.1)
        got = g.payload(0)
    finally:
        g.close()
    og = P.grid(res, res, res, bsx, st[1])
    slot = np.full(nb3, -1, np.int32)
    slot[bids] = np.arange(len(bids), dtype=np.int32)
    want = np.ascontiguousarray(init).copy()
    # ping-pong: the second buffer starts as a copy, so unlisted blocks read their values there
    P.pde(og, slot, np.ascontiguousarray(sub, np.int32), want, lt, 1, 3, 0.1, tmp=want.copy() if lt > 0 else None)
    assert np.array_equal(got.view(np.uint16 if storage == "u16" else np.uint32),
                          want.view(np.uint16 if storage == "u16" else np.uint32))
    unlisted = ~np.isin(bids, sub)
    assert np.array_equal(got[unlisted], init[unlisted])


def test_restriction_matches_reference_fixture(gpulib, port):
    G = gpulib
    gold = dict(np.load(os.path.join(GOLD, "reference_downsample.npz")))
    for nb, bsx, seed in H.DOWNSAMPLE_CASES:
        lv, st, pay = H.halo_case(nb, bsx, 3, seed, "f32", lambda *a: port.regularize(*a)[0])
        key = "x".join(map(str, nb)) + f"_bs{bsx}"
        g = G.MultiresSparseGrid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, 3, G.F32)
        try:
            g.set_levels(lv)
            g.setRefinementMap(0.0)
            for l in range(3):
                g.level_grid_set(0, l, G.F32, st[l], pay[l] if len(pay[l]) else None, H.DOWNSAMPLE_EMPTY,
                                 H.DOWNSAMPLE_FULL)
            bids = gold[f"{key}_bids"]
            for mode, simple in (("gauss", False), ("mean", True)):
                out, sk = g.restrict_level_blocks(0, 0, bids, simple)
                assert sk == 0
                assert np.array_equal(out.view(np.uint32), gold[f"{key}_{mode}"].view(np.uint32)), (key, mode)
        finally:
            g.close()


@pytest.mark.parametrize("storage,variant", [("f32", "exact"), ("f32", "fast"), ("u16", "exact")])
def test_surface512_full_size_matches_reference(gpulib, storage, variant):
    G = gpulib
    gold = dict(np.load(os.path.join(GOLD, "reference_surface512.npz")))
    spec = W.SURFACE_512
    pts = W.make_points(spec, 1)
    r = G.surface_pipeline(pts, spec["res"], spec["bsx"], storage={"f32": G.F32, "u16": G.U16}[storage],
                           n_iter=spec["n_iter"], dt=spec["dt"],
                           variant={"exact": G.SWEEP_EXACT, "fast": G.SWEEP_FAST}[variant])
    assert np.array_equal(r["active_bids"], gold["active_bids"])
    assert np.array_equal(r["levels"], gold["levels"]) and np.array_equal(r["flags"], gold["flags"])
    assert r["info"].nActParticles == int(gold["n_act_particles"])
    idx = gold["sample_index"]
    for stage, field in (("final", r["after_finalize"]), ("pde", r["after_pde"])):
        if storage == "f32":
            assert rel_l2(field.astype(np.float64).sum(1), gold[f"f32_{stage}_block_sums"]) < 1e-5
            assert rel_l2(field.reshape(-1)[idx], gold[f"f32_{stage}_sample"]) < 1e-5
        else:
            d = np.abs(field.reshape(-1)[idx].astype(np.int64) - gold[f"u16_{stage}_sample"].astype(np.int64))
            assert d.max() <= 8


def _multires_grid(G, nb, bsx, lv, x, b, dinv):
    """A context on the level map with level channels 0 = X, 1 = the diagonal channel, 2 = B:
    level l holds the blocks of level l (payload in ascending bid order), no block elsewhere."""
    g = G.MultiresSparseGrid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, 3, G.F32)
    g.set_levels(lv)
    g.setRefinementMap(0.0)
    off, spans = 0, []
    for l in range(3):
        at = lv == l
        st = np.full(lv.size, H.LBLK_NONE, np.int32)
        st[at] = np.arange(int(at.sum()), dtype=np.int32)
        n = int(at.sum()) * (bsx >> l) ** 3
        for lchan, arr in ((0, x), (1, dinv), (2, b)):
            g.level_grid_set(lchan, l, G.F32, st, arr[off:off + n] if n else None)
        spans.append((off, n))
        off += n
    return g, spans


@pytest.mark.parametrize("case", H.MULTIRES_CASES, ids=["x".join(map(str, c[0])) + f"_bs{c[1]}" for c in H.MULTIRES_CASES])
def test_multires_operator_matches_reference(gpulib, port, case):
    G = gpulib
    gold = dict(np.load(os.path.join(GOLD, "reference_multires.npz")))
    nb, bsx, seed = case
    key = "x".join(map(str, nb)) + f"_bs{bsx}"
    lv, x, b, dinv = H.multires_case(nb, bsx, 3, seed, lambda *a: port.regularize(*a)[0])
    assert np.array_equal(lv, gold[f"{key}_levels"])
    g, spans = _multires_grid(G, nb, bsx, lv, x, b, dinv)
    try:
        dot = 0.0
        for l, (off, n) in enumerate(spans):
            bids = np.flatnonzero(lv == l).astype(np.int32)
            y, d, sk = g.multiply_laplacian_levels(l, 0, 1, bids)
            assert sk == 0
            assert np.array_equal(y.reshape(-1).view(np.uint32), gold[f"{key}_y"][off:off + n].view(np.uint32)), (key, l)
            r, _, sk = g.multiply_laplacian_levels(l, 0, 1, bids, lchan_b=2, residual=True)
            assert sk == 0
            assert np.array_equal(r.reshape(-1).view(np.uint32), gold[f"{key}_r"][off:off + n].view(np.uint32)), (key, l)
            dot += d
        assert abs(dot - float(gold[f"{key}_dot"])) <= 1e-12 * abs(dot)
        # a block of another level, and one out of range, are skipped; the rest is unchanged
        bids0 = np.flatnonzero(lv == 0).astype(np.int32)
        other = np.flatnonzero(lv == 1)[:1].astype(np.int32)
        y, _, sk = g.multiply_laplacian_levels(0, 0, 1, np.concatenate([bids0, other, [lv.size]]).astype(np.int32))
        assert sk == 2
        off, n = spans[0]
        assert np.array_equal(y[: len(bids0)].reshape(-1).view(np.uint32), gold[f"{key}_y"][off:off + n].view(np.uint32))
        # an operand level channel that is not set
        with pytest.raises(G.MsbgGpuError) as e:
            g.multiply_laplacian_levels(0, 7, 1, bids0)
        assert e.value.code == G.ERR_STATE
    finally:
        g.close()


@pytest.mark.parametrize("case", H.MULTIRES_CASES, ids=["x".join(map(str, c[0])) + f"_bs{c[1]}" for c in H.MULTIRES_CASES])
def test_multires_block_smoother_matches_reference(gpulib, port, case):
    """msbg_gpu_relax_levels against relaxBlockList run by the reference: bit for bit, X relaxed
    in place in device arrays bound as level channel 3."""
    G = gpulib
    L = G.load_library()
    gold = dict(np.load(os.path.join(GOLD, "reference_multires.npz")))
    nb, bsx, seed = case
    key = "x".join(map(str, nb)) + f"_bs{bsx}"
    lv, x, b, dinv = H.multires_case(nb, bsx, 3, seed, lambda *a: port.regularize(*a)[0])
    g, spans = _multires_grid(G, nb, bsx, lv, x, b, dinv)
    bufs = []
    try:
        for l, (off, n) in enumerate(spans):
            at = lv == l
            st = np.full(lv.size, H.LBLK_NONE, np.int32)
            st[at] = np.arange(int(at.sum()), dtype=np.int32)
            ds, dp = g.to_device(st), g.to_device(x[off:off + n].copy() if n else np.zeros(4, np.float32))
            bufs += [ds, dp]
            g.level_grid_bind(3, l, G.F32, ds.ptr, dp.ptr)
        bids = np.arange(lv.size, dtype=np.int32)
        for passes, rev in H.MULTIRES_RELAX_RUNS:
            for l, (off, n) in enumerate(spans):  # X from the start
                if n:
                    src = np.ascontiguousarray(x[off:off + n])
                    assert L.msbg_gpu_copy_h2d(g.h, bufs[2 * l + 1].ptr, src.ctypes.data, src.nbytes) == 0
            for _ in range(passes):
                assert g.relax_levels(3, 2, 1, bids, reverse=rev) == 0
            got = np.empty_like(x)
            for l, (off, n) in enumerate(spans):
                if n:
                    assert L.msbg_gpu_copy_d2h(g.h, got[off:off + n].ctypes.data, bufs[2 * l + 1].ptr, 4 * n) == 0
            g.synchronize()
            want = gold[f"{key}_relaxed_{passes}_{int(rev)}"]
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (key, passes, rev)
        # out-of-range ids are skipped, once per call
        assert g.relax_levels(3, 2, 1, np.array([lv.size, -1], np.int32)) == 2
    finally:
        for d in bufs:
            d.free()
        g.close()


@pytest.mark.parametrize("case", H.DENSE_CASES, ids=[f"{c[0]}x{c[1]}x{c[2]}_L{c[4]}" for c in H.DENSE_CASES])
def test_dense_level_operator_matches_reference(gpulib, case):
    """msbg_gpu_multiply_laplacian_dense against the reference's operator at a dense multigrid
    level: bit for bit; cells of skipped groups keep what the output held."""
    G = gpulib
    gold = dict(np.load(os.path.join(GOLD, "reference_dense.npz")))
    sx0, sy0, sz0, bsx, nl, seed = case
    key = f"{sx0}x{sy0}x{sz0}_L{nl}"
    flags, x, b, dinv, ax, ay, az = H.dense_case(sx0, sy0, sz0, nl, seed)
    g = G.MultiresSparseGrid(sx0, sy0, sz0, bsx, nl, G.F32)
    try:
        y = g.multiply_laplacian_dense(nl, flags, x, dinv, ax, ay, az)
        assert np.array_equal(y.view(np.uint32), gold[f"{key}_y"].view(np.uint32))
        r = g.multiply_laplacian_dense(nl, flags, x, dinv, ax, ay, az, b=b, residual=True)
        assert np.array_equal(r.view(np.uint32), gold[f"{key}_r"].view(np.uint32))
        marker = np.full(flags.shape, 7.0, np.float32)
        y7 = g.multiply_laplacian_dense(nl, flags, x, dinv, ax, ay, az, y_init=marker)
        fluid = (flags & (H.CELL_SOLID | H.CELL_VOID)) == 0
        assert (y7[fluid] != 7.0).all()  # every fluid cell is written
        kept = y7 == 7.0  # cells of skipped groups, all non-fluid
        assert not fluid[kept].any() and np.array_equal(y7[~kept].view(np.uint32), y[~kept].view(np.uint32))
    finally:
        g.close()


@pytest.mark.parametrize("case", H.DENSE_CASES, ids=[f"{c[0]}x{c[1]}x{c[2]}_L{c[4]}" for c in H.DENSE_CASES])
def test_dense_level_smoother_matches_reference(gpulib, case):
    G = gpulib
    gold = dict(np.load(os.path.join(GOLD, "reference_dense.npz")))
    sx0, sy0, sz0, bsx, nl, seed = case
    key = f"{sx0}x{sy0}x{sz0}_L{nl}"
    flags, x, b, dinv, ax, ay, az = H.dense_case(sx0, sy0, sz0, nl, seed)
    g = G.MultiresSparseGrid(sx0, sy0, sz0, bsx, nl, G.F32)
    try:
        for it in H.DENSE_RELAX_ITERS:
            got = g.relax_dense(nl, it, flags, x, b, dinv, ax, ay, az)
            assert np.array_equal(got.view(np.uint32), gold[f"{key}_relaxed_{it}"].view(np.uint32)), it
    finally:
        g.close()
