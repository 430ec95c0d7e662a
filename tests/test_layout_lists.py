"""setRefinementMap's outputs beyond levels and flags (src/msbg.cpp:1428-2165): the block lists
_blocksExisting and _blocksFineCoarsePerLevel, and the fine-coarse distance channel
CH_DIST_FINECOARSE of every level (uint16(1024 d) per cell of a fine-coarse block, full blocks
around them).

CPU: the restatement bit for bit against the reference (fixture tests/golden/reference_layout.npz
on the 3- and 4-level maps of reference_small.npz, and fresh reference runs where the reference
is built here).  GPU: msbg_gpu_get_block_list and msbg_gpu_dist_fine_coarse bit for bit against
the fixture and the restatement."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT

LAYOUT_GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_layout.npz")
BLK_EXISTS, BLK_FINE_COARSE = 1 << 12, 1 << 3


@pytest.fixture(scope="module")
def lg():
    return dict(np.load(LAYOUT_GOLDEN))


def _check_dist(state, data, lg, nl, l):
    assert np.array_equal(np.nonzero(state >= 0)[0], lg[f"lvl{nl}_dist{l}_value_bids"])
    assert np.array_equal(data, lg[f"lvl{nl}_dist{l}_value"])
    assert np.array_equal(np.nonzero(state == -2)[0], lg[f"lvl{nl}_dist{l}_full_bids"])


def test_restatement_matches_reference_fixture(port, golden, lg):
    for nl in (3, 4):
        lv, flags = golden[f"lvl{nl}_out"].astype(np.int32), golden[f"lvl{nl}_flags"]
        assert np.array_equal(np.nonzero(flags & BLK_EXISTS)[0], lg[f"lvl{nl}_existing"])
        for l in range(nl):
            assert np.array_equal(np.nonzero((lv == l) & ((flags & BLK_FINE_COARSE) != 0))[0],
                                  lg[f"lvl{nl}_fine_coarse{l}"])
            state, data = port.dist_fine_coarse(lv, flags, (8, 8, 8), 16, l)
            _check_dist(state, data, lg, nl, l)
            assert int(lg[f"lvl{nl}_dist{l}_full_value"]) == 6 * 1024
    assert sum(len(lg[f"lvl4_dist{l}_full_bids"]) for l in range(4)) > 0


def test_restatement_matches_fresh_reference(port):
    import oracle_io as O
    if not O.ref_available():
        pytest.skip("the reference is not built on this host")
    rng = np.random.Generator(np.random.PCG64(20261203 + 990))
    nb, bsx, nl = (10, 7, 9), 16, 3
    u = rng.random(int(np.prod(nb)))
    lv = np.where(u < 0.05, 0, np.where(u < 0.15, 1, nl - 1)).astype(np.int32)
    lvr, _ = port.regularize(lv, *nb, nl)
    flags = port.block_flags(lvr, *nb)
    r = O.run_reference_layout(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, nl, lv)
    for l in range(nl):
        assert np.array_equal(np.nonzero((lvr == l) & ((flags & BLK_FINE_COARSE) != 0))[0], r["fine_coarse"][l])
        state, data = port.dist_fine_coarse(lvr, flags, nb, bsx, l)
        d = r["dist"][l]
        assert np.array_equal(np.nonzero(state >= 0)[0], d["value_bids"])
        assert np.array_equal(data, d["value"])
        assert np.array_equal(np.nonzero(state == -2)[0], d["full_bids"])


@pytest.mark.gpu
def test_gpu_matches_reference_fixture(gpulib, golden, lg):
    G = gpulib
    for nl in (3, 4):
        g = G.MultiresSparseGrid(128, 128, 128, 16, nl, G.F32)
        try:
            g.set_levels(golden[f"lvl{nl}_in"])
            g.regularizeRefinementMap()
            g.setRefinementMap(0.0)
            # The levels-only reference job allocates no channel data, so no block of it carries
            # BLK_EXISTS; this library gives every level-0 block its value block (and the bit).
            keep = np.uint16(0xFFFF & ~BLK_EXISTS)
            assert np.array_equal(g.flags() & keep, golden[f"lvl{nl}_flags"])
            assert len(lg[f"lvl{nl}_existing"]) == 0
            lv = golden[f"lvl{nl}_out"]
            assert np.array_equal(g.block_list(g.LIST_EXISTING), np.nonzero(lv == 0)[0])
            for l in range(nl):
                assert np.array_equal(g.block_list(g.LIST_FINE_COARSE, l), lg[f"lvl{nl}_fine_coarse{l}"])
                state, data = g.dist_fine_coarse(l)
                _check_dist(state, data, lg, nl, l)
        finally:
            g.close()


@pytest.mark.gpu
def test_gpu_existing_blocks_of_the_demo_pipeline(gpulib, golden):
    """_blocksExisting of the reference's demo pipeline (reference_small.npz: levels, flags and
    active blocks after setRefinementMap with value blocks) equals this library's list."""
    G = gpulib
    res, bsx = int(golden["res"]), int(golden["bsx"])
    want = np.nonzero(golden["flags"] & BLK_EXISTS)[0]
    assert np.array_equal(want, golden["active_bids"])
    g = G.MultiresSparseGrid(res, res, res, bsx, 3, G.F32)
    try:
        g.set_levels(golden["levels"].astype(np.int32))
        g.regularizeRefinementMap()
        g.setRefinementMap(0.0)
        assert np.array_equal(g.levels(), golden["levels"])
        assert np.array_equal(g.flags(), golden["flags"])
        assert np.array_equal(g.block_list(g.LIST_EXISTING), want)
    finally:
        g.close()
