"""Cross-resolution halo fill: HaloBlockSet::fillHaloBlock_<T> (src/halo.cpp:266-479) with
getOutOfBlockValue (src/halo.h:270-330) on a multi-level channel.

CPU: known answers of the restatement (interior = own block, Neumann clamp, the
coarse-level fallback at p/2 on level+1, the domain clamp before it), and the restatement
bit for bit against the reference's own fillHaloBlock_: the committed fixture
tests/golden/reference_halo.npz and, where the reference library was built here, fresh
layouts with 16^3 blocks.  GPU: msbg_gpu_fill_halo_blocks bit for bit against the same
fixture and against the restatement on larger seeded layouts (FP32, FP16, uint16; block
edges 32 and 16; halo sizes 1, 2, 4), plus skipped blocks and error codes."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT
import halo_cases as H

HALO_GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_halo.npz")
BC_NEUMANN, BC_COARSE_LEVEL = 1 << 10, 1 << 26
OPTS = (0, BC_NEUMANN, BC_COARSE_LEVEL)


@pytest.fixture(scope="module")
def hg():
    return dict(np.load(HALO_GOLDEN))


def _same(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.int32), np.asarray(b, np.float32).view(np.int32))


def _reg(port):
    return lambda *a: port.regularize(*a)[0]


def _fixture_case(hg, kind):
    nl = int(hg["n_levels"])
    return (hg[f"{kind}_levels"], [hg[f"{kind}_state{l}"] for l in range(nl)],
            [hg[f"{kind}_pay{l}"] for l in range(nl)])


def _port_storage(port, kind):
    return {"f32": port.F32, "u16": port.U16, "f16": port.F16}[kind]


def _host(pay):
    return [p.view(np.uint16) if p.dtype == np.float16 else p for p in pay]


# ---------------------------------------------------------------- CPU: restatement

def test_known_answers(port):
    """Two blocks of 8^3 along x on a 2-level channel.  Block 0 (level 0) holds v = x +
    10 y + 100 z; block 1 has no level-0 block and a constant 7 at level 1."""
    bs = 8
    g = port.grid(2 * bs, bs, bs, bs, port.F32)
    lv = np.array([0, 1], np.int32)
    own = (np.arange(bs)[None, None, :] + 10 * np.arange(bs)[None, :, None] +
           100 * np.arange(bs)[:, None, None]).astype(np.float32).reshape(1, -1)
    st0 = np.array([0, H.LBLK_NONE], np.int32)
    st1 = np.array([H.LBLK_EMPTY, 0], np.int32)
    pay1 = np.full((1, (bs // 2) ** 3), 7.0, np.float32)
    hs = bs + 2
    for opt in OPTS:
        out, sk = port.fill_halo(g, lv, [st0, st1], [own, pay1], 0, np.array([0], np.int32), 1, opt, 0.5, 1.0)
        assert sk == 0
        box = out.reshape(hs, hs, hs)
        assert np.array_equal(box[1:-1, 1:-1, 1:-1].ravel(), own.ravel())       # interior
        face = box[1:-1, 1:-1, -1]                                               # x = 8: block 1
        lowx = box[1:-1, 1:-1, 0]                                                # x = -1: outside
        if opt == BC_NEUMANN:
            assert np.array_equal(face, own.reshape(bs, bs, bs)[:, :, -1])
            assert np.array_equal(lowx, own.reshape(bs, bs, bs)[:, :, 0])
        elif opt == BC_COARSE_LEVEL:
            assert np.all(face == 7.0)                                           # level 1 at p/2
            assert np.array_equal(lowx, own.reshape(bs, bs, bs)[:, :, 0])        # clamped into block 0
        else:
            assert np.all(face == 0.5) and np.all(lowx == 0.5)                   # the empty value
    # a block at another level, or without a block at its level, is skipped
    _, sk = port.fill_halo(g, lv, [st0, st1], [own, pay1], 0, np.array([1], np.int32), 1, 0)
    assert sk == 1


def test_restatement_matches_reference_fixture(port, hg):
    nb, bsx, nl = tuple(int(v) for v in hg["nb"]), int(hg["bsx"]), int(hg["n_levels"])
    ev, fv = float(hg["empty_value"]), float(hg["full_value"])
    for kind in ("f32", "u16"):
        lv, st, pay = _fixture_case(hg, kind)
        g = port.grid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, _port_storage(port, kind))
        for L in range(nl):
            bids = H.blocks_at(lv, st, L)
            for opt in OPTS:
                for h in (1, 2):
                    out, sk = port.fill_halo(g, lv, st, pay, L, bids, h, opt, ev, fv)
                    assert sk == 0
                    assert _same(out, hg[f"{kind}_L{L}_o{opt}_h{h}"]), (kind, L, opt, h)


def test_restatement_matches_compiled_reference(port):
    import oracle_io as O
    if not O.ref_available():
        pytest.skip("reference library not built here (x86-64 build container only)")
    nb, bsx, nl = (5, 6, 4), 16, 3
    res = [v * bsx for v in nb]
    for kind, chan in (("f32", O.CHAN_F32), ("u16", O.CHAN_U16)):
        lv, st, pay = H.halo_case(nb, bsx, nl, 4100 + chan, kind, _reg(port))
        g = port.grid(*res, bsx, _port_storage(port, kind))
        for L in range(nl):
            for opt in OPTS:
                h = 1 + L % 2
                bids, ref = O.run_reference_halo(*res, bsx, nl, chan, lv, st, pay, L, h, opt, 0.0, 1.0)
                out, _ = port.fill_halo(g, lv, st, pay, L, bids, h, opt, 0.0, 1.0)
                assert _same(out, ref), (kind, L, opt)


# ---------------------------------------------------------------- GPU

def _gpu_grid(G, nb, bsx, nl, lv, st, pay, storage, ev=0.0, fv=1.0, lchan=0):
    g = G.MultiresSparseGrid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, nl, G.F32)
    g.set_levels(lv)
    g.setRefinementMap(0.0)
    for l in range(nl):
        g.level_grid_set(lchan, l, storage, st[l], pay[l] if len(pay[l]) else None, ev, fv)
    return g


@pytest.mark.gpu
def test_gpu_matches_reference_fixture(gpulib, hg):
    G = gpulib
    nb, bsx, nl = tuple(int(v) for v in hg["nb"]), int(hg["bsx"]), int(hg["n_levels"])
    ev, fv = float(hg["empty_value"]), float(hg["full_value"])
    for kind, storage in (("f32", G.F32), ("u16", G.U16)):
        lv, st, pay = _fixture_case(hg, kind)
        g = _gpu_grid(G, nb, bsx, nl, lv, st, pay, storage, ev, fv, lchan=3)
        try:
            for L in range(nl):
                bids = H.blocks_at(lv, st, L)
                for opt in OPTS:
                    for h in (1, 2):
                        out, sk = g.fill_halo_blocks(3, L, bids, h, opt)
                        ref = hg[f"{kind}_L{L}_o{opt}_h{h}"]
                        assert sk == 0
                        assert _same(out, ref), (kind, L, opt, h, int((out != ref).sum()))
        finally:
            g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["f32", "f16", "u16"])
@pytest.mark.parametrize("bsx", [16, 32])
def test_gpu_matches_restatement(gpulib, port, kind, bsx):
    """A seeded 3-level channel on an 8 x 7 x 9 block grid: every listed block of every
    level, all options, halo sizes 1, 2 and 4, bit for bit."""
    G = gpulib
    nb, nl = (8, 7, 9), 3
    lv, st, pay = H.halo_case(nb, bsx, nl, 5200 + bsx + len(kind), kind, _reg(port))
    storage = {"f32": G.F32, "f16": G.F16, "u16": G.U16}[kind]
    g = _gpu_grid(G, nb, bsx, nl, lv, st, pay, storage, 0.125, 0.875)
    try:
        og = port.grid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, _port_storage(port, kind))
        hp = _host(pay)
        for L in range(nl):
            bids = H.blocks_at(lv, st, L)
            assert len(bids) > 0
            for opt in OPTS:
                for h in (1, 2, 4):
                    if h > bsx >> L:
                        continue
                    out, sk = g.fill_halo_blocks(0, L, bids, h, opt)
                    ref, _ = port.fill_halo(og, lv, st, hp, L, bids, h, opt, 0.125, 0.875)
                    assert sk == 0
                    assert _same(out, ref), (kind, bsx, L, opt, h, int((out != ref).sum()))
    finally:
        g.close()


@pytest.mark.gpu
def test_gpu_fill_halo_skips_and_errors(gpulib, port):
    G = gpulib
    nb, bsx, nl = (4, 4, 4), 16, 3
    lv, st, pay = H.halo_case(nb, bsx, nl, 6100, "f32", _reg(port))
    g = G.MultiresSparseGrid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, nl, G.F32)
    try:
        with pytest.raises(G.MsbgGpuError) as e:  # no layout yet
            g.level_grid_set(0, 0, G.F32, st[0], pay[0])
            g.fill_halo_blocks(0, 0, np.array([0], np.int32), 1, 0)
        assert e.value.code == G.ERR_STATE
        g.set_levels(lv)
        g.setRefinementMap(0.0)
        with pytest.raises(G.MsbgGpuError) as e:  # level 1 never set
            g.fill_halo_blocks(0, 1, H.blocks_at(lv, st, 1), 1, 0)
        assert e.value.code == G.ERR_STATE
        for l in range(nl):
            g.level_grid_set(0, l, G.F32, st[l], pay[l])
        # a block of another level in the list is skipped, the others are filled
        b0, b1 = H.blocks_at(lv, st, 0), H.blocks_at(lv, st, 1)
        mixed = np.concatenate([b0, b1[:1]]).astype(np.int32)
        out, sk = g.fill_halo_blocks(0, 0, mixed, 1, BC_COARSE_LEVEL)
        ref, _ = port.fill_halo(port.grid(64, 64, 64, bsx, port.F32), lv, st, pay, 0, b0, 1, BC_COARSE_LEVEL)
        assert sk == 1
        assert _same(out[: len(b0)], ref)
        for bad in (dict(level=3), dict(level=-1)):
            with pytest.raises(G.MsbgGpuError) as e:
                g.fill_halo_blocks(0, bad["level"], b0, 1, 0)
            assert e.value.code == G.ERR_ARG
        with pytest.raises(G.MsbgGpuError) as e:  # halo wider than the level-2 block (4)
            g.fill_halo_blocks(0, 2, H.blocks_at(lv, st, 2), 5, 0)
        assert e.value.code == G.ERR_ARG
        with pytest.raises(G.MsbgGpuError) as e:  # OPT_INTERPOLATE (interpolateGhost)
            g.fill_halo_blocks(0, 0, b0, 1, BC_COARSE_LEVEL | (1 << 7))
        assert e.value.code == G.ERR_UNSUPPORTED
        bad_state = st[0].copy()
        bad_state[0] = len(pay[0])  # index past the payload
        with pytest.raises(G.MsbgGpuError) as e:
            g.level_grid_set(0, 0, G.F32, bad_state, pay[0])
        assert e.value.code == G.ERR_ARG
        assert g.L.msbg_gpu_fill_halo_blocks(g.h, 0, 0, None, 0, 1, 0, None, None) == G.OK
    finally:
        g.close()


# ---------------------------------------------------------------- restriction with the halo

def test_restrict_level_restatement_equals_value_block_restriction(port):
    """On a single-level layout (value blocks at level 0, every other block the constant empty
    block) the multi-level restriction is downsampleFloatChannelNew's value-block case."""
    rng = np.random.default_rng(3)
    res, bs = 96, 16
    nb3 = (res // bs) ** 3
    bids = np.nonzero(rng.random(nb3) < 0.5)[0].astype(np.int32)
    pay = rng.standard_normal((len(bids), bs ** 3)).astype(np.float32)
    slot = np.full(nb3, H.LBLK_EMPTY, np.int32)
    slot[bids] = np.arange(len(bids), dtype=np.int32)
    lv = np.full(nb3, 1, np.int32)
    lv[bids] = 0
    g = port.grid(res, res, res, bs, port.F32)
    for simple in (False, True):
        out, sk = port.restrict_level(g, lv, [slot, np.full(nb3, H.LBLK_NONE, np.int32)], [pay, None], 0, bids,
                                      simple)
        assert sk == 0
        assert _same(out, port.downsample(g, slot, bids, pay, simple)), simple


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["f32", "f16", "u16"])
def test_gpu_restrict_level_matches_restatement(gpulib, port, kind):
    G = gpulib
    storage = {"f32": G.F32, "f16": G.F16, "u16": G.U16}[kind]
    for bsx in (16, 32):
        nb, nl = (7, 6, 8), 3
        lv, st, pay = H.halo_case(nb, bsx, nl, 7300 + bsx + len(kind), kind, _reg(port))
        g = _gpu_grid(G, nb, bsx, nl, lv, st, pay, storage, 0.125, 0.875)
        try:
            og = port.grid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, _port_storage(port, kind))
            hp = _host(pay)
            for L in range(nl):
                bids = H.blocks_at(lv, st, L)
                for simple in (False, True):
                    out, sk = g.restrict_level_blocks(0, L, bids, simple)
                    ref, _ = port.restrict_level(og, lv, st, hp, L, bids, simple, 0.125, 0.875)
                    assert sk == 0
                    assert _same(out, ref), (kind, bsx, L, simple, int((out != ref).sum()))
        finally:
            g.close()


@pytest.mark.gpu
def test_gpu_restrict_level_equals_downsample_channel(gpulib):
    """Level 0 of a level channel bound to the value-block slab: the multi-level restriction
    equals msbg_gpu_downsample_channel bit for bit."""
    G = gpulib
    rng = np.random.default_rng(11)
    res, bs = 128, 16
    nb3 = (res // bs) ** 3
    bids = np.nonzero(rng.random(nb3) < 0.4)[0].astype(np.int32)
    pay = rng.standard_normal((len(bids), bs ** 3)).astype(np.float16)
    g = G.MultiresSparseGrid(res, res, res, bs, 2, G.F16)
    try:
        levels = np.full(nb3, 1, np.int32)
        levels[bids] = 0
        g.set_levels(levels)
        g.setRefinementMap(0.0)
        g.upload_payload(pay, 0)
        d_st = g.to_device(g.slots())  # -1 = the constant empty block, as in the value-block layout
        try:
            g.level_grid_bind(0, 0, G.F16, d_st.ptr, g.payload_ptr(0), 0.0, 1.0)
            g.level_grid_set(0, 1, G.F16, np.full(nb3, H.LBLK_NONE, np.int32), None)
            for simple in (False, True):
                out, _ = g.restrict_level_blocks(0, 0, g.active_blocks(), simple)
                assert _same(out, g.downsampleFloatChannelNew(0, simple)), simple
        finally:
            g.close()
            d_st.free()
    finally:
        g.close()


# ---------------------------------------------------------------- the solver's halo (fillHaloBlock3)

H3_GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_halo3.npz")


def _halo3_case(port, nb, bsx, seed):
    lv, st, pay = H.halo_case(nb, bsx, 3, seed, "f32", _reg(port))
    fst, fpay, ef, ff = H.flags_case(st, bsx, seed + 100)
    return lv, st, pay, fst, fpay, ef, ff


def test_halo3_restatement_matches_reference_fixture(port):
    """fillHaloBlock3 (src/halo.cpp:536-738): the restatement equals the reference bit for bit,
    markers (+1e20 void / open faces, -1e20 solid / closed faces) included."""
    gold = dict(np.load(H3_GOLDEN))
    for nb, bsx, seed, dbc in H.HALO3_CASES:
        lv, st, pay, fst, fpay, ef, ff = _halo3_case(port, nb, bsx, seed)
        key = "x".join(map(str, nb)) + f"_bs{bsx}"
        bids = gold[f"{key}_bids"]
        assert np.array_equal(bids, np.nonzero(lv == 0)[0])
        g = port.grid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, port.F32)
        out, sk = port.fill_halo3(g, lv, st, pay, fst, fpay, bids, dbc, H.DOWNSAMPLE_EMPTY, H.DOWNSAMPLE_FULL, ef, ff)
        assert sk == 0
        assert _same(out, gold[f"{key}_halo"]), key
        assert (np.abs(out) == 1e20).mean() > 0.05  # the markers are exercised


def test_halo3_restatement_matches_fresh_reference(port):
    import oracle_io as O
    if not O.ref_available():
        pytest.skip("the reference is not built on this host")
    nb, bsx, dbc = (3, 3, 2), 32, (0, 0, 1, 0, 0, 1)
    lv, st, pay, fst, fpay, ef, ff = _halo3_case(port, nb, bsx, 20261203 + 985)
    sx, sy, sz = (n * bsx for n in nb)
    bids, ref = O.run_reference_halo3(sx, sy, sz, bsx, 3, lv, st, pay, fst, fpay, dbc, 0.1, 0.9, ef, ff)
    g = port.grid(sx, sy, sz, bsx, port.F32)
    out, _ = port.fill_halo3(g, lv, st, pay, fst, fpay, bids, dbc, 0.1, 0.9, ef, ff)
    assert _same(out, ref)


@pytest.mark.gpu
def test_gpu_halo3_matches_reference_fixture_and_restatement(gpulib, port):
    G = gpulib
    gold = dict(np.load(H3_GOLDEN))
    cases = list(H.HALO3_CASES) + [((3, 3, 2), 32, 20261203 + 985, (0, 0, 1, 0, 0, 1))]
    for nb, bsx, seed, dbc in cases:
        lv, st, pay, fst, fpay, ef, ff = _halo3_case(port, nb, bsx, seed)
        g = _gpu_grid(G, nb, bsx, 3, lv, st, pay, G.F32, H.DOWNSAMPLE_EMPTY, H.DOWNSAMPLE_FULL, lchan=2)
        try:
            for l in range(3):
                g.level_flags_set(5, l, fst[l], fpay[l] if len(fpay[l]) else None, ef, ff)
            bids = np.nonzero(lv == 0)[0].astype(np.int32)
            # a block of another level in the list is skipped
            extra = np.nonzero(lv != 0)[0][:1].astype(np.int32)
            out, sk = g.fillHaloBlock3(2, 5, np.concatenate([bids, extra]), dbc)
            assert sk == len(extra)
            og = port.grid(nb[0] * bsx, nb[1] * bsx, nb[2] * bsx, bsx, port.F32)
            want, _ = port.fill_halo3(og, lv, st, pay, fst, fpay, bids, dbc, H.DOWNSAMPLE_EMPTY, H.DOWNSAMPLE_FULL,
                                      ef, ff)
            assert _same(out[: len(bids)], want), (nb, bsx)
            key = "x".join(map(str, nb)) + f"_bs{bsx}"
            if f"{key}_halo" in gold:
                assert _same(out[: len(bids)], gold[f"{key}_halo"]), key
        finally:
            g.close()
