"""GPU parity: the sm_103a library, called through its C ABI, against the CPU
oracles on identical seeded inputs.

* Against the reference's golden vectors (tests/golden): integer outputs bit for
  bit, fields within relative L2 1e-5.
* Against the CPU restatement: integer outputs bit for bit; FP32 / uint16 /
  FP16 / FP64 fields of the EXACT sweep variant bit for bit (same expression
  order, every operation rounded once); the FAST variant within rel-L2 1e-5.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2
from msbg_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
OPT8 = 1 << 29
MCF8 = -(4 + OPT8)
GOLDEN_NAMES = ["mcf8_f32", "mcf8_u16_odd", "jacobi_rb_f32", "jacobi_pp_f32_odd", "diff_pp_f32",
                "lapl8_f32", "pmj8_f32"]


def _gpu_pipeline(gpulib, pts, res, bsx, storage, n_iter, lapl_typ, dt, alpha=0.0, variant=0,
                  levels_in=None, bands=None, n_levels=3, constr01=1):
    G = gpulib
    sx, sy, sz = (res, res, res) if np.isscalar(res) else res
    g = G.MultiresSparseGrid(sx, sy, sz, bsx, n_levels, storage)
    try:
        d = g.to_device(np.ascontiguousarray(pts, np.float32))
        n = len(pts)
        if bands is not None:
            g.levels_from_bands(d, n, bands)
        else:
            g.mark_points(d, n, 4.0)
            g.levels_from_marks()
        if levels_in is not None:
            g.set_levels(levels_in)
        g.regularizeRefinementMap()
        g.setRefinementMap(1.0)
        g.splat(d, n, 2.0, 2.0)
        g.splat_finalize(2.0, 2.0)
        fin = g.payload(0)
        if n_iter:
            g.applyChannelPdeFast(0, laplTyp=lapl_typ, doConstrZeroOne=constr01, numIter=n_iter, timeStep=dt,
                                  anisDiffAlpha=alpha, variant=variant)
        out = dict(levels=g.levels(), flags=g.flags(), bids=g.active_blocks(), final=fin,
                   pde=g.payload(0), info=g.info(), launches=g.launch_count())
        d.free()
        return out
    finally:
        g.close()


def _as_bits(a):
    a = np.asarray(a)
    return a.view(np.uint16) if a.dtype == np.float16 else a


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_gpu_matches_reference_golden_and_port(gpulib, port, golden, name):
    chan, lt, it, dt, al = golden[f"meta_{name}"]
    storage = gpulib.F32 if int(chan) == 0 else gpulib.U16
    res, bsx = int(golden["res"]), int(golden["bsx"])
    r = _gpu_pipeline(gpulib, golden["points"], res, bsx, storage, int(it), int(lt), float(dt), float(al))
    assert np.array_equal(r["levels"], golden["levels"])
    assert np.array_equal(r["flags"], golden["flags"])
    assert np.array_equal(r["bids"], golden["active_bids"])
    assert r["info"].nActParticles == int(golden["n_act_particles"])
    want = golden[f"pde_{name}"]
    to_f = (lambda a: a) if storage == gpulib.F32 else (lambda a: port.to_float(port.U16, a))
    assert rel_l2(to_f(r["pde"]), to_f(want)) <= REL_TOL
    # bit-exact against the CPU restatement
    p = port.surface_pipeline(golden["points"], res, bsx, storage=storage, n_iter=int(it),
                              lapl_typ=int(lt), dt=float(dt), anis_alpha=float(al))
    assert np.array_equal(r["final"], p.after_finalize)
    assert np.array_equal(r["pde"], p.after_pde)
    assert r["launches"] > 0


def test_gpu_abort_rule(gpulib, port, golden):
    res, bsx = int(golden["res"]), int(golden["bsx"])
    r = _gpu_pipeline(gpulib, golden["points"], res, bsx, gpulib.F32, 2, MCF8, 0.1,
                      levels_in=golden["abort_levels_in"])
    assert np.array_equal(r["levels"], golden["abort_levels"])
    assert np.array_equal(r["bids"], golden["abort_active_bids"])
    assert rel_l2(r["final"], golden["abort_final_f32"]) <= REL_TOL
    assert rel_l2(r["pde"], golden["abort_pde_f32"]) <= REL_TOL
    p = port.surface_pipeline(golden["points"], res, bsx, storage=port.F32, n_iter=2, dt=0.1,
                              levels_in=golden["abort_levels_in"])
    assert r["info"].nAborted == p.n_aborted > 0
    assert np.array_equal(r["final"], p.after_finalize)
    assert np.array_equal(r["pde"], p.after_pde)


@pytest.mark.parametrize("nl", [3, 4])
def test_gpu_refinement_map_golden(gpulib, golden, nl):
    g = gpulib.MultiresSparseGrid(128, 128, 128, 16, nl, gpulib.F32)
    try:
        g.set_levels(golden[f"lvl{nl}_in"])
        g.regularizeRefinementMap()
        g.setRefinementMap(0.0)
        assert np.array_equal(g.levels(), golden[f"lvl{nl}_out"])
        fl = g.flags()
        # the demo's allocation loop adds BLK_EXISTS to level-0 blocks afterwards
        assert np.array_equal(fl & ~np.uint16(gpulib.BLK_EXISTS), golden[f"lvl{nl}_flags"])
        assert np.array_equal((fl & gpulib.BLK_EXISTS) != 0, golden[f"lvl{nl}_out"] == 0)
        per = np.array(g.info().blocksPerLevel[:])
        assert np.array_equal(per, golden[f"lvl{nl}_per_level"])
    finally:
        g.close()


@pytest.mark.parametrize("storage", ["F32", "U16", "F16", "F64"])
@pytest.mark.parametrize("bsx", [16, 32])
def test_gpu_vs_port_seeded(gpulib, port, storage, bsx):
    res = 256
    pts = W.sphere_cloud(res, 12, 6000, seed=W.workload_seed(1, 50 + bsx))
    st = getattr(gpulib, storage)
    r = _gpu_pipeline(gpulib, pts, res, bsx, st, 4, MCF8, 0.1)
    p = port.surface_pipeline(pts, res, bsx, storage=getattr(port, storage), n_iter=4, dt=0.1)
    assert np.array_equal(r["levels"], p.levels)
    assert np.array_equal(r["flags"], p.flags)
    assert np.array_equal(r["bids"], p.active_bids)
    assert np.array_equal(_as_bits(r["final"]), _as_bits(p.after_finalize))
    assert np.array_equal(_as_bits(r["pde"]), _as_bits(p.after_pde))


# FP32 storage: rel-L2 1e-5.  FP16 / uint16 storage: a result that the fast form
# rounds to the neighbouring storage value moves by one storage step (2^-11
# relative for FP16, 1/65535 for uint16), so the bound is 1e-3 there.
FAST_CASES = [("mcf", 16, "F32", 1, 1e-5), ("jacobi", 16, "F32", 1, 1e-5), ("mcf", 16, "F32", 0, 1e-5),
              ("mcf", 32, "F16", 1, 1e-3), ("jacobi", 32, "F16", 0, 1e-3), ("jacobi", 32, "U16", 1, 1e-3),
              ("mcf", 32, "F32", 1, 1e-5), ("jacobi", 32, "F32", 1, 1e-5), ("jacobi", 16, "F16", 1, 1e-3)]


@pytest.mark.parametrize("lapl,bsx,storage,constr01,tol", FAST_CASES)
def test_gpu_fast_variant_within_tolerance(gpulib, port, lapl, bsx, storage, constr01, tol):
    res = 256
    typ = MCF8 if lapl == "mcf" else -(17 + (1 << 29))
    pts = W.sphere_cloud(res, 12, 6000, seed=W.workload_seed(1, 77))
    r = _gpu_pipeline(gpulib, pts, res, bsx, getattr(gpulib, storage), 20, typ, 0.1,
                      variant=gpulib.SWEEP_FAST, constr01=constr01)
    p = port.surface_pipeline(pts, res, bsx, storage=getattr(port, storage), n_iter=20, dt=0.1,
                              lapl_typ=typ, constr01=constr01)
    assert np.array_equal(r["bids"], p.active_bids)

    def values(a):  # FP16 payloads: the restatement keeps the bit patterns
        a = np.asarray(a)
        if storage == "F16" and a.dtype == np.uint16:
            a = a.view(np.float16)
        return a.astype(np.float64)

    err = rel_l2(values(r["pde"]), values(p.after_pde))
    assert err <= tol, err
    moved = rel_l2(values(p.after_pde), values(p.after_finalize))
    assert moved > 100 * tol  # the sweeps really changed the field


def test_gpu_band_levels_vs_port(gpulib, port):
    res = 512
    pts = W.ellipsoid_cloud(res, 20, 3000, seed=W.workload_seed(2, 5), axis_range=(0.02, 0.08))
    r = _gpu_pipeline(gpulib, pts, res, 32, gpulib.F16, 2, MCF8, 0.1, bands=(8.0, 16.0))
    p = port.surface_pipeline(pts, res, 32, storage=port.F16, n_iter=2, dt=0.1, bands=(8.0, 16.0))
    assert np.array_equal(r["levels"], p.levels)
    assert set(np.unique(r["levels"])) == {0, 1, 2}
    assert np.array_equal(r["bids"], p.active_bids)
    assert np.array_equal(_as_bits(r["pde"]), _as_bits(p.after_pde))


def test_gpu_empty_and_out_of_domain_points(gpulib):
    pts = np.array([[-5.0, 3.0, 3.0], [70.0, 1.0, 1.0], [0.001, 30.0, 30.0]], np.float32)
    r = _gpu_pipeline(gpulib, pts, 64, 16, gpulib.F32, 2, MCF8, 0.1)
    assert r["info"].nActParticles == 0
    assert len(r["bids"]) == 0
    r = _gpu_pipeline(gpulib, np.zeros((0, 3), np.float32), 64, 16, gpulib.F32, 2, MCF8, 0.1)
    assert len(r["bids"]) == 0


def test_gpu_domain_boundary_neumann(gpulib, port):
    # a sphere that crosses the domain faces: marks clamp to the grid, the halo
    # falls back to the Neumann clamp outside the domain
    rng = np.random.Generator(np.random.PCG64(99))
    d = rng.standard_normal((4000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pts = (np.array([3.0, 60.0, 32.0]) + 10.0 * d).astype(np.float32)
    r = _gpu_pipeline(gpulib, pts, 64, 16, gpulib.F32, 4, MCF8, 0.1)
    p = port.surface_pipeline(pts, 64, 16, storage=port.F32, n_iter=4, dt=0.1)
    assert r["info"].nActParticles == p.n_act_particles < len(pts)
    assert np.array_equal(r["bids"], p.active_bids)
    assert np.array_equal(r["pde"], p.after_pde)


def test_gpu_surface_job_entry_point(gpulib):
    res = 128
    pts = W.sphere_cloud(res, 6, 3000, seed=W.workload_seed(1, 11))
    step = _gpu_pipeline(gpulib, pts, res, 16, gpulib.F32, 6, MCF8, 0.1)
    g = gpulib.MultiresSparseGrid(res, res, res, 16, 3, gpulib.F32)
    try:
        out = np.empty((res // 16) ** 3 * 16 ** 3, np.float32)
        n = g.surface_job(pts, numIter=6, timeStep=0.1, out=out)
        assert n == len(step["bids"])
        assert np.array_equal(out[: n * 4096].reshape(n, 4096), step["pde"])
    finally:
        g.close()


def test_gpu_surface_job_streaming_equals_one_at_a_time(gpulib):
    """msbg_gpu_surface_job_submit: a sequence of different jobs queued back to back (the next
    job's upload and this job's download overlap the compute) gives every job the result of
    msbg_gpu_surface_job, bit for bit, with FP16 and FP32 payloads."""
    G = gpulib
    res = 128
    clouds = [W.sphere_cloud(res, k, 2500, seed=W.workload_seed(1, 30 + k)) for k in (3, 6, 4, 5)]
    for storage, dt in ((G.F32, np.float32), (G.F16, np.float16)):
        nb3 = (res // 16) ** 3
        want = []
        g = G.MultiresSparseGrid(res, res, res, 16, 3, storage)
        try:
            for pts in clouds:
                out = np.zeros(nb3 * 4096, dt)
                n = g.surface_job(pts, numIter=6, timeStep=0.1, out=out)
                want.append((n, out.copy()))
        finally:
            g.close()
        g = G.MultiresSparseGrid(res, res, res, 16, 3, storage)
        try:
            outs = [np.full(nb3 * 4096, 7, dt) for _ in clouds]
            ns = [g.surface_job_submit(pts, out, numIter=6, timeStep=0.1) for pts, out in zip(clouds, outs)]
            g.surface_job_wait()
            for (n, w), m, out in zip(want, ns, outs):
                assert m == n
                assert np.array_equal(out[: n * 4096].view(np.uint8), w[: n * 4096].view(np.uint8))
        finally:
            g.close()


def test_gpu_error_codes(gpulib):
    G = gpulib
    with pytest.raises(G.MsbgGpuError) as e:
        G.MultiresSparseGrid(100, 64, 64, 16)
    with pytest.raises(G.MsbgGpuError) as e:
        G.MultiresSparseGrid(64, 64, 64, 12)
    g = G.MultiresSparseGrid(64, 64, 64, 16, 3, G.F32, capacity_blocks=2)
    try:
        with pytest.raises(G.MsbgGpuError) as e:
            g.applyChannelPdeFast(0, laplTyp=MCF8, doConstrZeroOne=1, numIter=2, timeStep=0.1)
        assert e.value.code == G.ERR_STATE
        pts = W.sphere_cloud(64, 2, 2000, seed=5, radius_range=(0.15, 0.2))
        d = g.to_device(pts)
        g.mark_points(d, len(pts), 4.0)
        g.levels_from_marks()
        with pytest.raises(G.MsbgGpuError) as e:
            g.setRefinementMap(1.0)
        assert e.value.code == G.ERR_CAPACITY
        d.free()
    finally:
        g.close()
    g = G.MultiresSparseGrid(64, 64, 64, 16, 3, G.F32)
    try:
        g.set_levels(np.zeros(64, np.int32))
        g.setRefinementMap(0.5)
        with pytest.raises(G.MsbgGpuError) as e:
            g.applyChannelPdeFast(0, laplTyp=-(2 + OPT8), doConstrZeroOne=1, numIter=2, timeStep=0.1)
        assert e.value.code == G.ERR_UNSUPPORTED
        with pytest.raises(G.MsbgGpuError) as e:
            g.set_levels(np.full(64, 7, np.int32))
        assert e.value.code == G.ERR_ARG
    finally:
        g.close()


def test_full_size_surface512_matches_restatement(gpulib, port):
    """The 512^3 surface workload at full size (64 spheres x 32,000 points, bs16,
    20 MCF iterations, FP32; EXACT sweep variant): active set, levels, flags and the
    particle counters bit for bit, the field after finalize and after the sweeps bit
    for bit as well (same expression order), against the CPU restatement."""
    spec = W.SURFACE_512
    pts = W.make_points(spec, 1)
    r = _gpu_pipeline(gpulib, pts, spec["res"], spec["bsx"], gpulib.F32, spec["n_iter"], MCF8, spec["dt"],
                      variant=gpulib.SWEEP_EXACT)
    p = port.surface_pipeline(pts, spec["res"], spec["bsx"], storage=port.F32, n_iter=spec["n_iter"],
                              dt=spec["dt"])
    assert np.array_equal(r["bids"], p.active_bids)
    assert np.array_equal(r["levels"], p.levels) and np.array_equal(r["flags"], p.flags)
    assert r["info"].nActParticles == p.n_act_particles and r["info"].nAborted == p.n_aborted
    assert np.array_equal(r["final"], p.after_finalize)
    assert np.array_equal(r["pde"], p.after_pde)
    assert len(r["bids"]) > 1000


def test_full_size_surface512_fp64_matches_restatement(gpulib, port):
    """The FP64 GPU path that the bench's field-error figure is measured against, at the
    512^3 workload's full size (FP64 storage and arithmetic, 4 MCF iterations, EXACT
    variant): bit for bit against the CPU FP64 restatement."""
    spec = W.SURFACE_512
    pts = W.make_points(spec, 1)
    r = _gpu_pipeline(gpulib, pts, spec["res"], spec["bsx"], gpulib.F64, 4, MCF8, spec["dt"],
                      variant=gpulib.SWEEP_EXACT)
    p = port.surface_pipeline(pts, spec["res"], spec["bsx"], storage=port.F64, n_iter=4, dt=spec["dt"])
    assert np.array_equal(r["bids"], p.active_bids)
    assert np.array_equal(_as_bits(r["final"]), _as_bits(p.after_finalize))
    assert np.array_equal(_as_bits(r["pde"]), _as_bits(p.after_pde))


def test_full_size_surface4096_layout_and_splat_match_restatement(gpulib, port):
    """The 4096^3 three-level FP16 workload at full size (1,024 clusters x 32,000
    points, bands 8 / 16 voxels): levels, flags, active set, particle counters and the
    FP16 field after splat + finalize, bit for bit against the CPU restatement."""
    spec = W.SURFACE_4096
    pts = W.make_points(spec, 2)
    bands = (spec["fine_band"], spec["mid_band"])
    r = _gpu_pipeline(gpulib, pts, spec["res"], spec["bsx"], gpulib.F16, 0, MCF8, spec["dt"], bands=bands,
                      n_levels=spec["n_levels"])
    p = port.surface_pipeline(pts, spec["res"], spec["bsx"], storage=port.F16, n_iter=0, bands=bands,
                              n_levels=spec["n_levels"])
    assert np.array_equal(r["bids"], p.active_bids)
    assert np.array_equal(r["levels"], p.levels) and np.array_equal(r["flags"], p.flags)
    assert r["info"].nActParticles == p.n_act_particles and r["info"].nAborted == p.n_aborted
    assert np.array_equal(_as_bits(r["final"]), _as_bits(p.after_finalize))
    assert len(r["bids"]) == 144191


def test_gpu_bounded_wait_times_out_and_context_stays_usable(gpulib):
    """The failure path of the library's bounded waits, without a GPU fault: a wait on
    an mbarrier that nothing completes gives up after its poll limit, the call returns
    MSBG_GPU_ERR_TIMEOUT, and the next calls on the same context work."""
    G = gpulib
    g = G.MultiresSparseGrid(64, 64, 64, 16, 2, G.F32)
    try:
        with pytest.raises(G.MsbgGpuError) as e:
            g.diag_wait_timeout(2000)
        assert e.value.code == G.ERR_TIMEOUT
        g.set_levels(np.zeros(64, np.int32))
        g.setRefinementMap(0.5)
        assert np.all(g.payload(0) == 0.5)
        with pytest.raises(G.MsbgGpuError) as e:  # the status word was cleared: same result again
            g.diag_wait_timeout(10)
        assert e.value.code == G.ERR_TIMEOUT
    finally:
        g.close()


@pytest.mark.gpu
def test_gpu_large_payload_copies_split_over_two_streams(gpulib):
    """Host transfers above 64 MiB go out in two halves on two streams (two copy engines);
    a 512 MiB FP32 channel makes the round trip unchanged."""
    G = gpulib
    g = G.MultiresSparseGrid(512, 512, 512, 16, 1, G.F32)
    try:
        g.set_levels(np.zeros(32 ** 3, np.int32))
        g.setRefinementMap(0.0)
        rng = np.random.Generator(np.random.PCG64(7))
        data = rng.random((32 ** 3, 16 ** 3), dtype=np.float32)
        assert data.nbytes > 64 << 20
        g.upload_payload(data, 0)
        assert np.array_equal(g.payload(0), data)
        g.fill(0.25, 0)
        assert np.all(g.payload(0) == 0.25)
    finally:
        g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("bsx", [16, 32])
def test_gpu_particles_per_block_match_restatement(gpulib, port, bsx):
    """msbg_gpu_particles_per_block against the restatement: the same offsets, and the same
    points in every list (the order inside a list is unspecified, as in the reference)."""
    res = 256
    pts = W.sphere_cloud(res, 12, 6000, seed=W.workload_seed(1, 91))
    pts = np.concatenate([pts, np.array([[-1.0, 5.0, 5.0], [300.0, 1.0, 1.0]], np.float32)])
    g = gpulib.MultiresSparseGrid(res, res, res, bsx, 3, gpulib.F32)
    try:
        d = g.to_device(pts)
        off, idx = g.particles_per_block(d, len(pts))
    finally:
        g.close()
    want_off, want_idx = port.particles_per_block(port.grid(res, res, res, bsx, port.F32), pts)
    assert np.array_equal(off, want_off)
    assert len(idx) == len(pts) - 2
    got = np.concatenate([np.sort(idx[off[b]:off[b + 1]]) for b in range(len(off) - 1)])
    assert np.array_equal(got, want_idx)


@pytest.mark.gpu
def test_gpu_splat_takes_the_minimum_with_the_fp32_channel(gpulib):
    """On an FP32 channel the splat takes the minimum with what the channel holds, as the
    demo's splat does (src/msbg_demo.cpp:624-628): filled with 0.5 instead of 1.0, the result
    is min(0.5, the splat over 1.0) voxel by voxel."""
    G = gpulib
    res = 128
    pts = W.sphere_cloud(res, 6, 3000, seed=W.workload_seed(1, 93))
    out = {}
    for fill in (1.0, 0.5):
        g = G.MultiresSparseGrid(res, res, res, 16, 3, G.F32)
        try:
            d = g.to_device(pts)
            g.mark_points(d, len(pts), 4.0)
            g.levels_from_marks()
            g.regularizeRefinementMap()
            g.setRefinementMap(fill)
            g.splat(d, len(pts), 2.0, 2.0)
            out[fill] = g.payload(0)
        finally:
            g.close()
    assert out[1.0].min() < 0.5 < out[1.0].max()
    assert np.array_equal(out[0.5], np.minimum(out[1.0], np.float32(0.5)))


@pytest.mark.gpu
def test_gpu_lists_and_splat_edge_cases(gpulib):
    """No points: every per-block list is empty and the splat leaves an FP32 channel as it
    was (the minimum with nothing); a bad argument to the tuner is an argument error."""
    G = gpulib
    g = G.MultiresSparseGrid(64, 64, 64, 16, 2, G.F32)
    try:
        g.set_levels(np.zeros(64, np.int32))
        g.setRefinementMap(0.5)
        d = G.DeviceBuffer.alloc(12)
        try:
            off, idx = g.particles_per_block(d, 0)
            assert len(idx) == 0 and not off.any()
            g.splat(d, 0, 2.0, 2.0)
        finally:
            d.free()
        assert np.all(g.payload(0) == 0.5)
        assert g.info().nAborted == 0
        with pytest.raises(G.MsbgGpuError) as e:
            g._check(g.L.msbg_gpu_poisson_tuning(g.h, 7, None, 0, None))
        assert e.value.code == G.ERR_ARG
    finally:
        g.close()
