"""Restriction to the next coarser multigrid level, downsampleFloatChannelNew
(src/msbg4.cpp:1035-1379): the CPU restatement's known answers (the 4^3 kernel of
src/grid.c:30-70 reproduces constants and linear ramps, empty neighbours and the
domain clamp of the OPT_BC_COARSE_LEVEL halo), and the GPU kernel bit for bit against
the restatement on seeded layouts for every storage type and block size."""
from __future__ import annotations

import numpy as np
import pytest

BS = 16


def _layout(port, nb, occupied, storage):
    g = port.grid(nb * BS, nb * BS, nb * BS, BS, storage)
    slot = np.full(nb ** 3, -1, np.int32)
    bids = np.sort(np.asarray(occupied, np.int32))
    slot[bids] = np.arange(len(bids), dtype=np.int32)
    return g, slot, bids


def _coords(bids, nb, bs):
    """Global fine coordinates (x, y, z) of every voxel, [nActive][bs^3] each."""
    v = np.arange(bs ** 3)
    vx, vy, vz = v % bs, (v // bs) % bs, v // (bs * bs)
    bx, by, bz = bids % nb, (bids // nb) % nb, bids // (nb * nb)
    return (bx[:, None] * bs + vx[None], by[:, None] * bs + vy[None], bz[:, None] * bs + vz[None])


def test_constant_and_linear_fields_are_reproduced(port):
    nb = 4
    g, slot, bids = _layout(port, nb, np.arange(nb ** 3), port.F32)  # every block holds data
    pay = np.full((len(bids), BS ** 3), 0.75, np.float32)
    for simple in (False, True):
        out = port.downsample(g, slot, bids, pay, simple)
        assert np.all(out == 0.75)
    # a ramp in x: the (1,3,3,1)/8 weights and the 2-child mean both give the coarse
    # cell centre 2v + 0.5, exactly, away from the clamped domain faces
    x, _, _ = _coords(bids, nb, BS)
    pay = x.astype(np.float32)
    cb = BS // 2
    c = np.arange(cb ** 3)
    cx = (bids % nb)[:, None] * cb + (c % cb)[None]
    inner = (cx > 0) & (cx < nb * cb - 1)
    for simple in (False, True):
        out = port.downsample(g, slot, bids, pay, simple)
        assert np.array_equal(out[inner], (2 * cx + 0.5)[inner].astype(np.float32))


def test_empty_neighbours_and_domain_clamp(port):
    nb = 3
    centre = 1 + nb + nb * nb  # block (1,1,1), surrounded by empty blocks
    g, slot, bids = _layout(port, nb, [centre], port.F32)
    pay = np.ones((1, BS ** 3), np.float32)
    out = port.downsample(g, slot, bids, pay).reshape(BS // 2, BS // 2, BS // 2)
    # corner coarse cell: in each axis the fine cell at -1 is empty -> (7/8)^3
    assert out[0, 0, 0] == np.float32(343 / 512)
    assert out[3, 3, 3] == 1.0 and out[0, 3, 3] == np.float32(7 / 8)
    assert np.all(port.downsample(g, slot, bids, pay, True) == 1.0)
    # block (0,0,0) alone: cells outside the domain clamp to the block (value 1),
    # the empty neighbour beyond x = bs gives 7/8 on that side
    g, slot, bids = _layout(port, nb, [0], port.F32)
    out = port.downsample(g, slot, bids, pay).reshape(BS // 2, BS // 2, BS // 2)
    assert out[0, 0, 0] == 1.0
    assert out[0, 0, BS // 2 - 1] == np.float32(7 / 8)
    assert out[BS // 2 - 1, BS // 2 - 1, BS // 2 - 1] == np.float32((7 / 8) ** 3)


def _random_layout(G, rng, res, bs, storage):
    g = G.MultiresSparseGrid(res, res, res, bs, 2, storage)
    nb = res // bs
    levels = np.where(rng.random(nb ** 3) < 0.35, 0, 1).astype(np.int32)
    levels[0] = 0  # a block at the domain corner
    levels[-1] = 0
    g.set_levels(levels)
    g.regularizeRefinementMap()
    g.setRefinementMap(0.0)
    n = g.info().nActive
    if storage == G.F32:
        pay = rng.standard_normal((n, bs ** 3)).astype(np.float32)
    elif storage == G.F16:
        pay = rng.standard_normal((n, bs ** 3)).astype(np.float16)
    else:
        pay = rng.integers(0, 65536, (n, bs ** 3)).astype(np.uint16)
    g.upload_payload(pay, 0)
    return g, pay


@pytest.mark.gpu
@pytest.mark.parametrize("bs", [16, 32])
@pytest.mark.parametrize("storage", ["F32", "F16", "U16"])
def test_gpu_matches_restatement(gpulib, port, bs, storage):
    G = gpulib
    rng = np.random.default_rng(1000 + bs)
    res = 128 if bs == 16 else 192
    g, pay = _random_layout(G, rng, res, bs, getattr(G, storage))
    try:
        bids = g.active_blocks().astype(np.int32)
        slot = g.slots().astype(np.int32)
        og = port.grid(res, res, res, bs, getattr(port, storage))
        host = pay.view(np.uint16) if storage == "F16" else pay
        for simple in (False, True):
            ref = port.downsample(og, slot, bids, host, simple)
            out = g.downsampleFloatChannelNew(0, simple)
            assert out.shape == ref.shape
            assert np.array_equal(out, ref), (simple, np.abs(out - ref).max())
    finally:
        g.close()


@pytest.mark.gpu
def test_gpu_downsample_errors(gpulib):
    G = gpulib
    g = G.MultiresSparseGrid(64, 64, 64, 16, 2, G.F64)
    try:
        with pytest.raises(G.MsbgGpuError) as e:  # no layout yet
            g.downsampleFloatChannelNew(0)
        assert e.value.code == G.ERR_STATE
        g.set_levels(np.zeros(64, np.int32))
        g.setRefinementMap(0.0)
        with pytest.raises(G.MsbgGpuError) as e:
            g.downsampleFloatChannelNew(0)
        assert e.value.code == G.ERR_UNSUPPORTED
        with pytest.raises(G.MsbgGpuError) as e:
            g.downsampleFloatChannelNew(5)
        assert e.value.code == G.ERR_ARG
    finally:
        g.close()
