"""The allocation-free slot assignment (msbg_gpu_assign_slots_noalloc).

It serves callers that cannot allocate device memory: its only scratch is a
fixed array inside the library.  This test calls it through the C ABI on
caller-owned device buffers and checks it against the slots and active-block
list that msbg_gpu_set_refinement_map builds, on two calls in a row (the
second call reuses the scratch the first one left behind).  It lives in a file
that pytest collects last and passes both alone and after the other tests.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(L, nbytes):
    p = C.c_void_p()
    assert L.msbg_gpu_device_alloc(C.byref(p), max(nbytes, 8)) == 0
    return p


def _reference_slots(G, levels, nb):
    g = G.MultiresSparseGrid(nb[0] * 16, nb[1] * 16, nb[2] * 16, 16, 3, G.F32)
    try:
        g.set_levels(levels)
        g.setRefinementMap(0.0)
        return g.slots(), g.active_blocks()
    finally:
        g.close()


def test_noalloc_slots_match_set_refinement_map(gpulib):
    G = gpulib
    L = G.load_library()
    nb = (40, 24, 32)
    n = int(np.prod(nb))
    rng = np.random.Generator(np.random.PCG64(20261203 + 77))
    maps = [rng.integers(0, 3, n).astype(np.int32),
            np.where(rng.random(n) < 0.03, 0, 2).astype(np.int32)]
    h = C.c_void_p()  # any context provides the copy helpers; the entry point itself needs none
    assert L.msbg_gpu_create(C.byref(h), 64, 64, 64, 16, 3, G.F32, 0) == 0
    d_lv, d_slot, d_act, d_cnt = (_dev(L, n * 4), _dev(L, n * 4), _dev(L, n * 4), _dev(L, 8))
    try:
        for lv in maps:  # two calls in a row share the scratch array
            assert L.msbg_gpu_copy_h2d(h, d_lv, lv.ctypes.data_as(C.c_void_p), lv.nbytes) == 0
            assert L.msbg_gpu_synchronize(h) == 0
            rc = L.msbg_gpu_assign_slots_noalloc(d_lv, n, d_slot, d_act, d_cnt, None)
            assert rc == 0
            cnt = np.zeros(1, np.int64)
            slot = np.empty(n, np.int32)
            assert L.msbg_gpu_copy_d2h(h, cnt.ctypes.data_as(C.c_void_p), d_cnt, 8) == 0
            assert L.msbg_gpu_copy_d2h(h, slot.ctypes.data_as(C.c_void_p), d_slot, n * 4) == 0
            act = np.empty(max(int(cnt[0]), 1), np.int32)
            assert L.msbg_gpu_copy_d2h(h, act.ctypes.data_as(C.c_void_p), d_act, int(cnt[0]) * 4) == 0
            want_slot, want_act = _reference_slots(G, lv, nb)
            assert int(cnt[0]) == len(want_act) == int((lv == 0).sum())
            assert np.array_equal(slot, want_slot)
            assert np.array_equal(act[: int(cnt[0])], want_act)
        # an empty map launches only the offsets kernel, which writes a count of 0
        junk = np.array([12345], np.int64)
        assert L.msbg_gpu_copy_h2d(h, d_cnt, junk.ctypes.data_as(C.c_void_p), 8) == 0
        assert L.msbg_gpu_synchronize(h) == 0
        assert L.msbg_gpu_assign_slots_noalloc(d_lv, 0, d_slot, d_act, d_cnt, None) == 0
        cnt = np.ones(1, np.int64)
        assert L.msbg_gpu_copy_d2h(h, cnt.ctypes.data_as(C.c_void_p), d_cnt, 8) == 0
        assert int(cnt[0]) == 0
        # oversized maps are refused before any launch
        too_big = G.load_library().msbg_gpu_assign_slots_noalloc(
            d_lv, (1 << 24) + 1, d_slot, d_act, d_cnt, None)
        assert too_big == G.ERR_CAPACITY
    finally:
        for p in (d_lv, d_slot, d_act, d_cnt):
            L.msbg_gpu_device_free(p)
        L.msbg_gpu_destroy(h)


def test_noalloc_slots_beyond_one_offset_chunk(gpulib):
    """About 2.2 M blocks: more than 512 scan tiles of 4,096 blocks, so the single-CTA
    offsets kernel carries its running total from one 512-tile chunk to the next.  The
    expectation comes from numpy: slots from the cumulative count of level-0 blocks and
    the active list from their indices."""
    G = gpulib
    L = G.load_library()
    n = 2_200_000
    rng = np.random.Generator(np.random.PCG64(20261203 + 78))
    lv = np.where(rng.random(n) < 0.2, 0, 1).astype(np.int32)
    want_act = np.flatnonzero(lv == 0).astype(np.int32)
    want_slot = np.where(lv == 0, np.cumsum(lv == 0) - 1, -1).astype(np.int32)
    h = C.c_void_p()
    assert L.msbg_gpu_create(C.byref(h), 64, 64, 64, 16, 3, G.F32, 0) == 0
    d_lv, d_slot, d_act, d_cnt = (_dev(L, n * 4), _dev(L, n * 4), _dev(L, n * 4), _dev(L, 8))
    try:
        assert L.msbg_gpu_copy_h2d(h, d_lv, lv.ctypes.data_as(C.c_void_p), lv.nbytes) == 0
        assert L.msbg_gpu_synchronize(h) == 0
        for _ in range(2):
            assert L.msbg_gpu_assign_slots_noalloc(d_lv, n, d_slot, d_act, d_cnt, None) == 0
            cnt = np.zeros(1, np.int64)
            slot = np.empty(n, np.int32)
            assert L.msbg_gpu_copy_d2h(h, cnt.ctypes.data_as(C.c_void_p), d_cnt, 8) == 0
            assert L.msbg_gpu_copy_d2h(h, slot.ctypes.data_as(C.c_void_p), d_slot, n * 4) == 0
            act = np.empty(len(want_act), np.int32)
            assert L.msbg_gpu_copy_d2h(h, act.ctypes.data_as(C.c_void_p), d_act, act.nbytes) == 0
            assert int(cnt[0]) == len(want_act)
            assert np.array_equal(slot, want_slot)
            assert np.array_equal(act, want_act)
    finally:
        for p in (d_lv, d_slot, d_act, d_cnt):
            L.msbg_gpu_device_free(p)
        L.msbg_gpu_destroy(h)
