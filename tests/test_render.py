"""Ray-march render of the iso-0.5 surface: RDR::RaymarchRenderer (src/render.h:52-160,
src/render.cpp:20-101), the demo's visual check of the density (src/msbg_demo.cpp:129-175).

CPU: the restatement against the reference's own renderer (fixture
tests/golden/reference_render.npz: the golden uint16 MCF field, two cameras, two image
sizes; fresh cameras where the reference library was built here).  The reference is built
with -ffast-math, so its normal and normalisation arithmetic may round a little differently:
hit masks must agree exactly, and at most 0.2% of the pixels may differ, by one step of one
colour channel.  GPU: msbg_gpu_render bit for bit against the restatement (both use the same
rounded operations), and within the same tolerance of the fixture."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT

RENDER_GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_render.npz")
MISS = 0x02000000
CAMERAS = {
    "demo": {"pos": (0.5, 0.8, 0.7), "look_at": (0.5, 0.5, 0.5), "sun": (0.5, 5.0, 5.0),
             "color": (0.8, 0.6, 0.4), "zoom": 1.0},
    "close": {"pos": (0.2, 0.55, 0.15), "look_at": (0.45, 0.45, 0.5), "sun": (-2.0, 3.0, -1.0),
              "color": (1.0, 1.0, 1.0), "zoom": 1.7},
}


@pytest.fixture(scope="module")
def rg():
    return dict(np.load(RENDER_GOLDEN))


def _rgb(px):
    """BMP_MKRGB int pixels -> uint8 [h][w][3] (r, g, b)."""
    px = np.asarray(px, np.int64)
    return np.stack([px & 255, (px >> 8) & 255, (px >> 16) & 255], -1).astype(np.uint8)


def _close(out_rgb, ref_px, frac=0.002):
    ref = _rgb(ref_px)
    hit_ref = np.asarray(ref_px) != MISS
    hit_out = out_rgb.any(-1) | hit_ref  # a hit may shade to black; compare where either hits
    d = np.abs(out_rgb.astype(np.int16) - ref.astype(np.int16)).max(-1)
    assert int(d.max()) <= 1, int(d.max())
    assert (d > 0).mean() <= frac, float((d > 0).mean())
    return int((d > 0).sum()), int(hit_out.sum())


def _scene(golden):
    res, bs = int(golden["res"]), int(golden["bsx"])
    bids = golden["active_bids"]
    slot = np.full((res // bs) ** 3, -1, np.int32)
    slot[bids] = np.arange(len(bids), dtype=np.int32)
    return res, bs, bids, slot, golden["pde_mcf8_u16_odd"]


# ---------------------------------------------------------------- CPU: restatement

def test_restatement_matches_reference_fixture(port, rg, golden):
    res, bs, _, slot, pay = _scene(golden)
    g = port.grid(res, res, res, bs, port.U16)
    for name, cam in CAMERAS.items():
        for w, h in ((160, 90), (320, 180)):
            ref = rg[f"{name}_{w}x{h}"]
            out = port.render(g, slot, pay, w, h, cam)
            assert np.array_equal(out != MISS, ref != MISS), (name, w, h)
            _close(_rgb(out), ref)


def test_restatement_matches_compiled_reference(port, golden):
    import oracle_io as O
    if not O.ref_available():
        pytest.skip("reference library not built here (x86-64 build container only)")
    res, bs, bids, slot, pay = _scene(golden)
    g = port.grid(res, res, res, bs, port.U16)
    rng = np.random.default_rng(31)
    for k in range(3):
        cam = {"pos": tuple(rng.uniform(0.0, 1.0, 3)), "look_at": tuple(rng.uniform(0.35, 0.65, 3)),
               "sun": tuple(rng.uniform(-5, 5, 3)), "color": tuple(rng.uniform(0.2, 1.0, 3)),
               "zoom": float(rng.uniform(0.7, 2.0))}
        ref, _, _ = O.run_reference_render(res, res, res, bs, bids, pay, 200, 150, cam)
        out = port.render(g, slot, pay, 200, 150, cam)
        assert np.array_equal(out != MISS, ref != MISS), k
        _close(_rgb(out), ref)


def test_restatement_known_answers(port):
    """An empty grid renders black; a grid full of density 1 seen from inside the domain is
    hit at the first step whose density reaches 0.5 and shaded by the sun."""
    g = port.grid(64, 64, 64, 16, port.U16)
    slot = np.full(64, -1, np.int32)
    out = port.render(g, slot, np.zeros((1, 16 ** 3), np.uint16), 40, 30)
    assert np.all(out == MISS)
    slot = np.arange(64, dtype=np.int32)
    full = np.full((64, 16 ** 3), 65535, np.uint16)
    out = port.render(g, slot, full, 40, 30)
    # the demo camera sits inside the domain, where the density is already 1: no ray
    # crosses 0.5 upwards before it leaves the domain
    assert np.all(out == MISS)


# ---------------------------------------------------------------- GPU

def _gpu_scene(G, res, bs, bids, pay, storage):
    g = G.MultiresSparseGrid(res, res, res, bs, 2, storage)
    levels = np.full((res // bs) ** 3, 1, np.int32)
    levels[np.asarray(bids)] = 0
    g.set_levels(levels)
    g.setRefinementMap(0.0)
    g.upload_payload(pay, 0)
    return g


@pytest.mark.gpu
def test_gpu_matches_reference_fixture_and_restatement(gpulib, port, rg, golden):
    G = gpulib
    res, bs, bids, slot, pay = _scene(golden)
    g = _gpu_scene(G, res, bs, bids, pay, G.U16)
    og = port.grid(res, res, res, bs, port.U16)
    try:
        for name, cam in CAMERAS.items():
            for w, h in ((160, 90), (320, 180)):
                out = g.render(0, w, h, cam)
                _close(out, rg[f"{name}_{w}x{h}"])
                assert np.array_equal(out, _rgb(port.render(og, slot, pay, w, h, cam))), (name, w, h)
    finally:
        g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["U16", "F32", "F16"])
def test_gpu_matches_restatement_512(gpulib, port, storage):
    """The 512^3 surface workload (64 spheres, 2.05 M points, 20 MCF sweeps) rendered at
    480x270 from the demo camera and from the close camera: bit for bit."""
    G = gpulib
    from msbg_gb300 import workloads as W
    pts = W.make_points(W.SURFACE_512, 1)
    st = getattr(G, storage)
    r = G.surface_pipeline(pts, 512, 16, storage=st, n_iter=20, lapl_typ=-(4 + (1 << 29)), dt=0.1)
    bids, pay = r["active_bids"], r["after_pde"]
    g = _gpu_scene(G, 512, 16, bids, pay, st)
    og = port.grid(512, 512, 512, 16, getattr(port, storage))
    slot = np.full(32 ** 3, -1, np.int32)
    slot[bids] = np.arange(len(bids), dtype=np.int32)
    host = pay.view(np.uint16) if storage == "F16" else pay
    try:
        for cam in CAMERAS.values():
            out = g.render(0, 480, 270, cam)
            ref = _rgb(port.render(og, slot, host, 480, 270, cam))
            assert out.any()
            assert np.array_equal(out, ref), int((out != ref).any(-1).sum())
    finally:
        g.close()


@pytest.mark.gpu
def test_gpu_render_errors(gpulib):
    G = gpulib
    g = G.MultiresSparseGrid(64, 64, 64, 16, 2, G.U16)
    try:
        with pytest.raises(G.MsbgGpuError) as e:  # no layout yet
            g.render(0, 8, 8)
        assert e.value.code == G.ERR_STATE
        g.set_levels(np.zeros(64, np.int32))
        g.setRefinementMap(0.0)
        buf = G.DeviceBuffer.alloc(8 * 8 * 3)
        try:
            for w, h in ((0, 8), (8, -1)):
                with pytest.raises(G.MsbgGpuError) as e:
                    g.render_device(0, w, h, CAMERAS["demo"], buf)
                assert e.value.code == G.ERR_ARG
        finally:
            buf.free()
        with pytest.raises(G.MsbgGpuError) as e:
            g.render(7, 8, 8)
        assert e.value.code == G.ERR_ARG
        assert np.all(g.render(0, 16, 8) == 0)  # a field of zeros: nothing crosses 0.5
    finally:
        g.close()
