"""Morton order of block lists: MultiresSparseGrid::sortBlockListMorton (src/msbg2.cpp:46-58)
with FMA::morton64_encode (src/fastmath.h:290-316).

CPU: the restatement's key against hand-computed interleavings, and the restatement's
order bit for bit against the reference's own sort (fixture tests/golden/reference_morton.npz,
and fresh lists where the reference library was built here).  GPU: msbg_gpu_sort_block_list_morton
against the fixture and the restatement, on cubic and elongated block grids, and its errors."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT

MORTON_GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_morton.npz")


@pytest.fixture(scope="module")
def mg():
    return dict(np.load(MORTON_GOLDEN))


def _grids(mg):
    for k in mg:
        if k.startswith("in_"):
            nb = tuple(int(v) for v in k[3:].split("x"))
            yield nb, mg[k], mg["out_" + k[3:]]


def test_key_interleaves_bits(port):
    assert port.lib().orc_morton64(1, 0, 0) == 1
    assert port.lib().orc_morton64(0, 1, 0) == 2
    assert port.lib().orc_morton64(0, 0, 1) == 4
    assert port.lib().orc_morton64(3, 5, 6) == sum(((3 >> b & 1) << 3 * b) | ((5 >> b & 1) << 3 * b + 1) |
                                                   ((6 >> b & 1) << 3 * b + 2) for b in range(3))
    assert port.lib().orc_morton64(0x1fffff, 0, 0) == 0x1249249249249249


def test_restatement_matches_reference_fixture(port, mg):
    for nb, bids, ref in _grids(mg):
        assert np.array_equal(port.sort_blocks_morton(*nb, bids), ref), nb


def test_restatement_matches_compiled_reference(port):
    import oracle_io as O
    if not O.ref_available():
        pytest.skip("reference library not built here (x86-64 build container only)")
    rng = np.random.default_rng(77)
    for nb in ((64, 64, 64), (7, 31, 2)):
        n = int(np.prod(nb))
        bids = rng.permutation(n)[: n // 2].astype(np.int32)
        ref = O.run_reference_morton(nb[0] * 8, nb[1] * 8, nb[2] * 8, 8, bids)
        assert np.array_equal(port.sort_blocks_morton(*nb, bids), ref), nb


@pytest.mark.gpu
def test_gpu_matches_reference_and_restatement(gpulib, port, mg):
    G = gpulib
    for nb, bids, ref in _grids(mg):
        g = G.MultiresSparseGrid(nb[0] * 16, nb[1] * 16, nb[2] * 16, 16, 2, G.F32)
        try:
            assert np.array_equal(g.sortBlockListMorton(bids), ref), nb
        finally:
            g.close()
    rng = np.random.default_rng(91)
    for nb in ((128, 128, 128), (100, 37, 64)):
        g = G.MultiresSparseGrid(nb[0] * 8, nb[1] * 8, nb[2] * 8, 8, 2, G.F32)
        try:
            n = int(np.prod(nb))
            for frac in (1.0, 0.1):
                bids = rng.permutation(n)[: int(n * frac)].astype(np.int32)
                assert np.array_equal(g.sortBlockListMorton(bids), port.sort_blocks_morton(*nb, bids)), (nb, frac)
        finally:
            g.close()


@pytest.mark.gpu
def test_gpu_morton_errors(gpulib):
    G = gpulib
    g = G.MultiresSparseGrid(64, 64, 64, 16, 2, G.F32)
    try:
        for bad in (np.array([3, 5, 3], np.int32), np.array([0, 64], np.int32), np.array([-1, 2], np.int32)):
            with pytest.raises(G.MsbgGpuError) as e:
                g.sortBlockListMorton(bad)
            assert e.value.code == G.ERR_ARG
        assert g.sortBlockListMorton(np.array([], np.int32)).size == 0
        assert np.array_equal(g.sortBlockListMorton(np.array([9], np.int32)), [9])
    finally:
        g.close()
