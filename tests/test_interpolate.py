"""Grid-to-particle trilinear interpolation: interpolateFloatFast (src/sbg.h:4623-4792),
interpolateUint16ToFloatFast (src/sbg.h:4920-5032) and interpolateRenderDensity
(src/msbg.h:478-484), with the generic border path interpolateGen0<IP_LINEAR>
(src/sbg.h:3109-3246).

CPU: the restatement's known answers (voxel centres give voxel values, linear fields are
reproduced, empty blocks read 0, the Dirichlet border options), and the restatement bit
for bit against the reference's own outputs: the committed fixture
tests/golden/reference_interp.npz and, where the reference library was built here, fresh
seeded points.  GPU: the kernel bit for bit against the same fixture and against the
restatement on larger seeded layouts, for FP32, uint16 and FP16 storage."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT

INTERP_GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_interp.npz")
IP_CORNER, IP_BC_DIRICHLET, IP_BC_DIRICHLET_OLD = 1 << 0, 1 << 13, 1 << 14
IP_NO_BORDER_CHECK, IP_RENDER_DENS = 1 << 15, 1 << 18
OPTS = (0, IP_CORNER, IP_BC_DIRICHLET, IP_BC_DIRICHLET_OLD, IP_CORNER | IP_BC_DIRICHLET, IP_RENDER_DENS)


@pytest.fixture(scope="module")
def ig():
    return dict(np.load(INTERP_GOLDEN))


def _slot(nb3, bids):
    slot = np.full(nb3, -1, np.int32)
    slot[np.asarray(bids)] = np.arange(len(bids), dtype=np.int32)
    return slot


def _rand_payloads(ig):
    u16 = ig["rand_u16"]
    f32 = (u16.astype(np.float32) * np.float32(1.0 / 65536.0)).astype(np.float32)
    return {"f32": f32, "u16": u16}


def _same(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.int32), np.asarray(b, np.float32).view(np.int32))


# ---------------------------------------------------------------- CPU: restatement

def test_voxel_centres_linear_fields_and_empty_blocks(port):
    res, bs = 32, 8
    nb = res // bs
    bids = np.arange(nb ** 3, dtype=np.int32)
    g = port.grid(res, res, res, bs, port.F32)
    v = np.arange(bs ** 3)
    x = (bids % nb)[:, None] * bs + (v % bs)[None]
    y = ((bids // nb) % nb)[:, None] * bs + ((v // bs) % bs)[None]
    z = (bids // (nb * nb))[:, None] * bs + (v // (bs * bs))[None]
    pay = (0.25 * x + 0.5 * y - 0.125 * z + 3.0).astype(np.float32)
    rng = np.random.default_rng(7)
    pts = rng.uniform(0.5, res - 0.5, (5000, 3)).astype(np.float32)
    out = port.interpolate(g, _slot(nb ** 3, bids), pay, pts)
    p = pts.astype(np.float64) - 0.5
    want = 0.25 * p[:, 0] + 0.5 * p[:, 1] - 0.125 * p[:, 2] + 3.0
    assert np.max(np.abs(out - want)) < 1e-4
    # a voxel centre returns the stored value exactly (t = 0)
    cen = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)[::97].astype(np.float32) + np.float32(0.5)
    assert _same(port.interpolate(g, _slot(nb ** 3, bids), pay, cen), pay.ravel()[::97])
    # one block with payload 1 in an empty grid: its interior is 1, halfway into the
    # empty neighbour along x is 1/2, inside an empty block 0
    one = np.ones((1, bs ** 3), np.float32)
    centre = 1 + nb + nb * nb
    s = _slot(nb ** 3, [centre])
    q = np.array([[12.0, 12.0, 12.0], [bs * 2 + 0.0, 12.0, 12.0], [28.0, 28.0, 28.0]], np.float32)
    assert _same(port.interpolate(g, s, one, q), [1.0, 0.5, 0.0])


def test_border_options(port):
    res, bs = 16, 8
    g = port.grid(res, res, res, bs, port.F32)
    bids = np.arange(8, dtype=np.int32)
    pay = np.full((8, bs ** 3), 2.0, np.float32)
    s = _slot(8, bids)
    q = np.array([[0.25, 8.0, 8.0], [15.9, 8.0, 8.0], [-3.0, -3.0, 40.0]], np.float32)
    assert _same(port.interpolate(g, s, pay, q), [2.0, 2.0, 2.0])           # clamped corners
    assert _same(port.interpolate(g, s, pay, q, IP_BC_DIRICHLET_OLD), [0.0, 0.0, 0.0])
    # Dirichlet: clipped corners read 0; at x = 0.25, t = 0.75 of the way from the
    # clipped corner (-1) to voxel 0
    d = port.interpolate(g, s, pay, q, IP_BC_DIRICHLET)
    assert d[0] == np.float32(1.5) and d[2] == 0.0


def test_restatement_matches_reference_fixture(port, ig, golden):
    pays = _rand_payloads(ig)
    res, bs = int(ig["rand_res"]), int(ig["rand_bsx"])
    slot = _slot((res // bs) ** 3, ig["rand_bids"])
    for name, st in (("f32", port.F32), ("u16", port.U16)):
        g = port.grid(res, res, res, bs, st)
        for opt in OPTS:
            key = f"rand_{name}_{opt}"
            if key not in ig:
                continue
            out = port.interpolate(g, slot, pays[name], ig["rand_points"], opt)
            assert _same(out, ig[key]), (key, int((out != ig[key]).sum()))
    res, bs = int(golden["res"]), int(golden["bsx"])
    slot = _slot((res // bs) ** 3, golden["active_bids"])
    for name, st, key in (("f32", port.F32, "pde_mcf8_f32"), ("u16", port.U16, "pde_mcf8_u16_odd")):
        g = port.grid(res, res, res, bs, st)
        for opt in (0, IP_RENDER_DENS):
            k = f"surf_{name}_{opt}"
            if k in ig:
                assert _same(port.interpolate(g, slot, golden[key], golden["points"], opt), ig[k]), k


def test_restatement_matches_compiled_reference(port):
    import oracle_io as O
    if not O.ref_available():
        pytest.skip("reference library not built here (x86-64 build container only)")
    res, bs = 64, 16
    nb3 = (res // bs) ** 3
    rng = np.random.default_rng(2026)
    bids = np.nonzero(rng.random(nb3) < 0.7)[0].astype(np.int32)
    slot = _slot(nb3, bids)
    pts = rng.uniform(-2.0, res + 2.0, (40000, 3)).astype(np.float32)
    pts[:10000] = np.floor(pts[:10000]) + np.float32(0.5)
    pays = {O.CHAN_F32: rng.standard_normal((len(bids), bs ** 3)).astype(np.float32),
            O.CHAN_U16: rng.integers(0, 65536, (len(bids), bs ** 3)).astype(np.uint16)}
    for chan, st in ((O.CHAN_F32, port.F32), (O.CHAN_U16, port.U16)):
        g = port.grid(res, res, res, bs, st)
        for opt in OPTS:
            if chan == O.CHAN_F32 and opt & IP_RENDER_DENS:
                continue
            ref, _, _ = O.run_reference_interp(res, res, res, bs, chan, bids, pays[chan], pts, opt)
            assert _same(port.interpolate(g, slot, pays[chan], pts, opt), ref), (chan, opt)


# ---------------------------------------------------------------- GPU

def _gpu_grid(G, res, bs, storage, bids, pay, n_levels=2):
    g = G.MultiresSparseGrid(res, res, res, bs, n_levels, storage)
    nb3 = (res // bs) ** 3
    levels = np.full(nb3, n_levels - 1, np.int32)
    levels[np.asarray(bids)] = 0
    g.set_levels(levels)
    g.setRefinementMap(0.0)
    assert np.array_equal(g.active_blocks(), np.sort(bids))
    g.upload_payload(pay, 0)
    return g


@pytest.mark.gpu
def test_gpu_matches_reference_fixture(gpulib, ig, golden):
    G = gpulib
    pays = _rand_payloads(ig)
    res, bs = int(ig["rand_res"]), int(ig["rand_bsx"])
    for name, st in (("f32", G.F32), ("u16", G.U16)):
        g = _gpu_grid(G, res, bs, st, ig["rand_bids"], pays[name])
        try:
            for opt in OPTS:
                key = f"rand_{name}_{opt}"
                if key not in ig:
                    continue
                out = g.interpolate(0, ig["rand_points"], opt)
                assert _same(out, ig[key]), (key, int((out != ig[key]).sum()))
        finally:
            g.close()
    res, bs = int(golden["res"]), int(golden["bsx"])
    for name, st, key in (("f32", G.F32, "pde_mcf8_f32"), ("u16", G.U16, "pde_mcf8_u16_odd")):
        g = _gpu_grid(G, res, bs, st, golden["active_bids"], golden[key], n_levels=3)
        try:
            for opt in (0, IP_RENDER_DENS):
                k = f"surf_{name}_{opt}"
                if k in ig:
                    assert _same(g.interpolate(0, golden["points"], opt), ig[k]), k
        finally:
            g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["F32", "F16", "U16"])
@pytest.mark.parametrize("bs", [16, 32])
def test_gpu_matches_restatement_large(gpulib, port, storage, bs):
    """A 512^3 layout with a third of the blocks holding data, 4 M points spread over
    the domain and its border (a quarter on block upper faces): every value bit for bit."""
    G = gpulib
    res = 512
    nb3 = (res // bs) ** 3
    rng = np.random.default_rng(4242 + bs)
    bids = np.nonzero(rng.random(nb3) < 0.33)[0].astype(np.int32)
    if storage == "F32":
        pay = rng.standard_normal((len(bids), bs ** 3)).astype(np.float32)
    elif storage == "F16":
        pay = rng.standard_normal((len(bids), bs ** 3)).astype(np.float16)
    else:
        pay = rng.integers(0, 65536, (len(bids), bs ** 3)).astype(np.uint16)
    n = 4_000_000
    pts = rng.uniform(-1.0, res + 1.0, (n, 3)).astype(np.float32)
    q = n // 4
    pts[:q, 1] = (rng.integers(0, res // bs, q) * bs + bs - 0.5 + rng.uniform(0, 1, q)).astype(np.float32)
    g = _gpu_grid(G, res, bs, getattr(G, storage), bids, pay)
    try:
        og = port.grid(res, res, res, bs, getattr(port, storage))
        host = pay.view(np.uint16) if storage == "F16" else pay
        slot = _slot(nb3, bids)
        for opt in (0, IP_RENDER_DENS | IP_BC_DIRICHLET):
            out = g.interpolate(0, pts, opt)
            ref = port.interpolate(og, slot, host, pts, opt)
            assert _same(out, ref), (opt, int((out != ref).sum()))
    finally:
        g.close()


@pytest.mark.gpu
def test_gpu_interpolate_errors(gpulib):
    G = gpulib
    g = G.MultiresSparseGrid(64, 64, 64, 16, 2, G.F32)
    try:
        with pytest.raises(G.MsbgGpuError) as e:  # no layout yet
            g.interpolate(0, np.zeros((4, 3), np.float32))
        assert e.value.code == G.ERR_STATE
        g.set_levels(np.zeros(64, np.int32))
        g.setRefinementMap(0.0)
        with pytest.raises(G.MsbgGpuError) as e:
            g.interpolate(0, np.zeros((4, 3), np.float32), 1 << 7)  # OPT_IPEXTRAPOL
        assert e.value.code == G.ERR_UNSUPPORTED
        with pytest.raises(G.MsbgGpuError) as e:
            g.interpolate(9, np.zeros((4, 3), np.float32))
        assert e.value.code == G.ERR_ARG
        assert g.L.msbg_gpu_interpolate(g.h, 0, None, -1, None, 0) == G.ERR_ARG
        assert g.L.msbg_gpu_interpolate(g.h, 0, None, 0, None, 0) == G.OK
        assert g.interpolate(0, np.zeros((0, 3), np.float32)).shape == (0,)
        # every supported option together is accepted
        opt = IP_CORNER | (1 << 5) | IP_BC_DIRICHLET | IP_BC_DIRICHLET_OLD | IP_NO_BORDER_CHECK | IP_RENDER_DENS
        out = g.interpolate(0, np.full((3, 3), 8.0, np.float32), opt)
        assert out.shape == (3,)
    finally:
        g.close()
