"""Checkpoint files (msbg_gpu_save / msbg_gpu_load): the reference has no on-disk format for its
grids (VDB writers declared only, src/sbg.h:599-605), so the file is this library's raw dump
of geometry, level map and channel payloads, each with an FNV-1a 64 checksum.

CPU: the documented layout, written by hand, read by the index reader.  GPU: save -> load
restores layout and payloads bit for bit, the restored grid sweeps exactly like the
original, and damaged files (payload byte, truncation, magic, missing file) are refused."""
from __future__ import annotations

import os
import struct

import numpy as np
import pytest


def _fnv(b: bytes) -> int:
    h = 0xcbf29ce484222325
    for x in b:
        h = ((h ^ x) * 0x100000001b3) & 0xffffffffffffffff
    return h


def test_index_reader_follows_the_documented_layout(tmp_path):
    from msbg_gb300 import gpu as G
    levels = np.array([0, 1, 2, 0, 1, 2, 2, 0], np.int8)
    pay0 = np.arange(3 * 8, dtype=np.float32).tobytes()
    pay5 = np.arange(3 * 8, dtype=np.uint16).tobytes()
    blob = struct.pack("<8sII6i2qQ", b"MSBGCKP1", 1, 64, 4, 4, 2, 2, 3, 2, 8, 3, _fnv(levels.tobytes()))
    blob += levels.tobytes()
    blob += struct.pack("<iiqQ", 0, G.F32, len(pay0), _fnv(pay0)) + pay0
    blob += struct.pack("<iiqQ", 5, G.U16, len(pay5), _fnv(pay5)) + pay5
    p = tmp_path / "x.msbg"
    p.write_bytes(blob)
    idx = G.read_checkpoint_index(str(p))
    assert (idx["sx"], idx["bsx"], idx["n_levels"], idx["n_blocks"], idx["n_active"]) == (4, 2, 3, 8, 3)
    assert [c["chan"] for c in idx["channels"]] == [0, 5]
    c5 = idx["channels"][1]
    assert c5["storage"] == G.U16 and c5["checksum"] == _fnv(pay5)
    assert blob[c5["offset"]:c5["offset"] + c5["bytes"]] == pay5
    p.write_bytes(b"MSBGCKP2" + blob[8:])
    with pytest.raises(ValueError):
        G.read_checkpoint_index(str(p))


def _grid(G):
    from msbg_gb300 import workloads as W
    spec = dict(W.SURFACE_512, res=256, n_objects=24, pts_per_object=8000)
    pts = W.make_points(spec, 1)
    g = G.MultiresSparseGrid(256, 256, 256, 16, 3, G.F16)
    d = g.to_device(pts)
    g.mark_points(d, len(pts), 4.0)
    g.levels_from_marks()
    g.regularizeRefinementMap()
    g.setRefinementMap(1.0)
    g.splat(d, len(pts), 2.0, 2.0)
    g.splat_finalize(2.0, 2.0)
    g.applyChannelPdeFast(0, laplTyp=G.LAPL_MCF_8COLOR, doConstrZeroOne=1, numIter=4, timeStep=0.1, variant=G.SWEEP_FAST)
    d.free()
    g.channel_create(3, G.F32)
    g.upload_payload(np.random.default_rng(3).standard_normal(
        (g.info().nActive, 16 ** 3)).astype(np.float32), 3)
    return g


@pytest.mark.gpu
def test_gpu_save_load_round_trip(gpulib, tmp_path):
    G = gpulib
    g = _grid(G)
    path = str(tmp_path / "grid.msbg")
    try:
        g.save(path, (0, 3))
        idx = G.read_checkpoint_index(path)
        h = G.MultiresSparseGrid.load(path)
        try:
            assert h.info().nActive == g.info().nActive == idx["n_active"]
            assert np.array_equal(h.levels(), g.levels())
            assert np.array_equal(h.flags(), g.flags())
            assert np.array_equal(h.active_blocks(), g.active_blocks())
            assert np.array_equal(h.slots(), g.slots())
            for chan in (0, 3):
                a, b = g.payload(chan), h.payload(chan)
                assert a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8)), chan
                rec = [c for c in idx["channels"] if c["chan"] == chan][0]
                with open(path, "rb") as f:
                    f.seek(rec["offset"])
                    raw = np.frombuffer(f.read(rec["bytes"]), a.dtype).reshape(a.shape)
                assert np.array_equal(raw.view(np.uint8), a.view(np.uint8))
            # the restored grid continues exactly as the original
            for x in (g, h):
                x.applyChannelPdeFast(0, laplTyp=G.LAPL_MCF_8COLOR, doConstrZeroOne=1, numIter=2, timeStep=0.1, variant=G.SWEEP_FAST)
            assert np.array_equal(g.payload(0).view(np.uint16), h.payload(0).view(np.uint16))
        finally:
            h.close()
    finally:
        g.close()


@pytest.mark.gpu
def test_gpu_checkpoint_errors(gpulib, tmp_path):
    G = gpulib
    g = _grid(G)
    path = str(tmp_path / "grid.msbg")
    try:
        with pytest.raises(G.MsbgGpuError) as e:
            g.save(path, (0, 7))  # channel 7 does not exist
        assert e.value.code == G.ERR_ARG
        with pytest.raises(G.MsbgGpuError) as e:
            g.save(str(tmp_path / "no" / "such" / "dir.msbg"))
        assert e.value.code == G.ERR_IO
        g.save(path, (0,))
        blob = bytearray(open(path, "rb").read())
        rec = G.read_checkpoint_index(path)["channels"][0]
        damaged = {"payload": blob[:rec["offset"] + 100] + bytes([blob[rec["offset"] + 100] ^ 1]) +
                   blob[rec["offset"] + 101:],
                   "truncated": blob[:-5], "magic": b"XSBGCKP1" + blob[8:],
                   "levels": blob[:70] + bytes([blob[70] ^ 1]) + blob[71:]}
        for name, b in damaged.items():
            p = str(tmp_path / f"{name}.msbg")
            open(p, "wb").write(bytes(b))
            with pytest.raises(G.MsbgGpuError) as e:
                G.MultiresSparseGrid.load(p)
            assert e.value.code == G.ERR_IO, name
        with pytest.raises(G.MsbgGpuError) as e:
            G.MultiresSparseGrid.load(str(tmp_path / "missing.msbg"))
        assert e.value.code == G.ERR_IO
    finally:
        g.close()


def _two_record_file(G, recs) -> bytes:
    """A 32^3 grid of 16^3 blocks with two value blocks, and the given (chan, storage, payload)
    records, each with a correct checksum."""
    levels = np.array([0, 1, 2, 0, 1, 2, 2, 2], np.int8)
    blob = struct.pack("<8sII6i2qQ", b"MSBGCKP1", 1, 64, 32, 32, 32, 16, 3, len(recs), 8, 2,
                       _fnv(levels.tobytes()))
    blob += levels.tobytes()
    for chan, storage, pay in recs:
        blob += struct.pack("<iiqQ", chan, storage, len(pay), _fnv(pay)) + pay
    return blob


@pytest.mark.gpu
def test_gpu_checkpoint_rejects_a_repeated_channel(gpulib, tmp_path):
    """A file that holds two records for one channel (here FP32 and then FP16 for channel 0,
    each consistent with its own storage type) is refused with MSBG_GPU_ERR_IO; copying both
    would write the FP32 record's bytes into a slab sized for FP16.  The same file with the
    records on two channels loads, and save refuses a channel listed twice."""
    G = gpulib
    p32 = np.arange(2 * 16 ** 3, dtype=np.float32).tobytes()
    p16 = np.arange(2 * 16 ** 3, dtype=np.float16).tobytes()
    bad = tmp_path / "dup.msbg"
    bad.write_bytes(_two_record_file(G, [(0, G.F32, p32), (0, G.F16, p16)]))
    with pytest.raises(G.MsbgGpuError) as e:
        G.MultiresSparseGrid.load(str(bad))
    assert e.value.code == G.ERR_IO
    good = tmp_path / "two.msbg"
    good.write_bytes(_two_record_file(G, [(0, G.F32, p32), (1, G.F16, p16)]))
    h = G.MultiresSparseGrid.load(str(good))
    try:
        assert h.info().nActive == 2
        assert h.payload(0).tobytes() == p32 and h.payload(1).tobytes() == p16
        with pytest.raises(G.MsbgGpuError) as e:
            h.save(str(tmp_path / "again.msbg"), (0, 1, 0))
        assert e.value.code == G.ERR_ARG
    finally:
        h.close()
