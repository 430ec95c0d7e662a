"""Regenerates the golden fixtures of tests/golden/ from the MSBG reference itself.

The reference library is compiled from its own sources by ``make -C oracle ref``
(x86-64 only) and driven by oracle/_ref/msbg_ref_driver, which runs the demo's
marking/splat/finalize loops and the library's regularizeRefinementMap,
setRefinementMap and applyChannelPdeFast<T> (see oracle/ref_driver.cpp).
This script needs the reference sources, so it runs in the build container,
never on the GPU host; the .npz files it writes are committed.

    python tests/golden/make_golden.py

It writes reference_small.npz (splat, levels, sweeps), reference_interp.npz
(trilinear interpolation), reference_halo.npz (cross-resolution halo fill),
reference_render.npz (ray-march render), reference_morton.npz (Morton-ordered block
lists), reference_solver.npz (the solver building blocks and the block smoother),
reference_downsample.npz (downsampleFloatChannelNew on multi-level channels) and
reference_surface512.npz (the 512^3 surface workload at full size: layout, counters,
per-block sums and a voxel sample of the fields), reference_halo3.npz (the solver's halo,
fillHaloBlock3), reference_layout.npz (setRefinementMap's block lists and fine-coarse
distance channel), reference_multires.npz (the solver operator and block smoother on
multi-resolution layouts) and reference_dense.npz (the operator at a dense multigrid
level).  Arguments name a subset
(small interp halo render morton solver downsample surface512 halo3 layout multires dense).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle_io as O  # noqa: E402

OPT8 = 1 << 29
RES, BSX = 64, 16


def golden_points() -> np.ndarray:
    """Two seeded spheres (radii 9 and 12 voxels) in a 64^3 grid, 1500 points each."""
    rng = np.random.Generator(np.random.PCG64(20261203 + 900))
    out = []
    for c, r in (((22.3, 25.1, 30.7), 9.0), ((40.2, 37.9, 33.4), 12.0)):
        d = rng.standard_normal((1500, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        out.append(np.asarray(c) + r * d + rng.normal(0, 0.1, (1500, 3)))
    return np.concatenate(out).astype(np.float32)


# (name, storage, laplTyp, numIter, dt, anisAlpha)
SWEEP_CASES = [
    ("mcf8_f32", O.CHAN_F32, -(4 + OPT8), 4, 0.1, 0.0),
    ("mcf8_u16_odd", O.CHAN_U16, -(4 + OPT8), 5, 0.1, 0.0),
    ("jacobi_rb_f32", O.CHAN_F32, -17, 3, 0.1, 0.0),
    ("jacobi_pp_f32_odd", O.CHAN_F32, 17, 3, 0.1, 0.0),
    ("diff_pp_f32", O.CHAN_F32, 3, 2, 0.2, 0.0),
    ("lapl8_f32", O.CHAN_F32, -(1 + OPT8), 2, 0.1, 0.0),
    ("pmj8_f32", O.CHAN_F32, -(15 + OPT8), 2, 0.1, 0.2),
]


def main(which: list[str]) -> None:
    if not O.ref_available():
        raise SystemExit("oracle/_ref/msbg_ref_driver missing: run `make -C oracle ref` first")
    parts = set(which) or {"small", "interp", "halo", "render", "morton", "solver", "downsample", "surface512",
                           "halo3", "layout", "multires", "dense"}
    if parts & {"small", "interp", "render"}:
        out = make_small()
        if "interp" in parts:
            make_interp(out)
        if "render" in parts:
            make_render(out)
    if "halo" in parts:
        make_halo()
    if "morton" in parts:
        make_morton()
    if "solver" in parts:
        make_solver()
    if "downsample" in parts:
        make_downsample()
    if "surface512" in parts:
        make_surface512()
    if "halo3" in parts:
        make_halo3()
    if "layout" in parts:
        make_layout()
    if "multires" in parts:
        make_multires()
    if "dense" in parts:
        make_dense()


def make_small() -> dict:
    pts = golden_points()
    out = {"points": pts, "res": np.int32(RES), "bsx": np.int32(BSX)}
    for name, chan, lt, it, dt, al in SWEEP_CASES:
        r = O.run_reference_surface(O.SurfaceJob(RES, RES, RES, BSX, pts, chan=chan, n_iter=it,
                                                 lapl_typ=lt, dt=dt, anis_alpha=al))
        if "levels" not in out:
            out["levels"] = r.levels
            out["flags"] = r.flags
            out["active_bids"] = r.active_bids
            out["n_act_particles"] = np.int64(r.n_act_particles)
        else:
            assert np.array_equal(out["levels"], r.levels)
        if chan == O.CHAN_F32 and "final_f32" not in out:
            out["final_f32"] = r.after_finalize
        if chan == O.CHAN_U16 and "final_u16" not in out:
            out["final_u16"] = r.after_finalize
        out[f"pde_{name}"] = r.after_pde
        out[f"meta_{name}"] = np.array([chan, lt, it, dt, al], np.float64)

    # abort rule: a fifth of the active blocks forced to level 1
    nb = (RES // BSX) ** 3
    lv = out["levels"].astype(np.int32).copy()
    rng = np.random.Generator(np.random.PCG64(20261203 + 901))
    act = np.nonzero(lv == 0)[0]
    lv[rng.choice(act, max(1, len(act) // 5), replace=False)] = 1
    r = O.run_reference_surface(O.SurfaceJob(RES, RES, RES, BSX, pts, chan=O.CHAN_F32, n_iter=2,
                                             dt=0.1, levels=lv))
    out["abort_levels_in"] = lv
    out["abort_levels"] = r.levels
    out["abort_active_bids"] = r.active_bids
    out["abort_final_f32"] = r.after_finalize
    out["abort_pde_f32"] = r.after_pde
    assert nb == lv.size

    # multi-level refinement maps (regularize + BlockInfo flags), 8^3 blocks
    for nl in (3, 4):
        rng = np.random.Generator(np.random.PCG64(20261203 + 910 + nl))
        u = rng.random(8 ** 3)
        lv = np.where(u < 0.04, 0, np.where(u < 0.10, 1, nl - 1)).astype(np.int32)
        r = O.run_reference_levels(8 * BSX, 8 * BSX, 8 * BSX, BSX, nl, lv)
        out[f"lvl{nl}_in"] = lv
        out[f"lvl{nl}_out"] = r.levels
        out[f"lvl{nl}_flags"] = r.flags
        out[f"lvl{nl}_per_level"] = r.blocks_per_level

    path = os.path.join(HERE, "reference_small.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")
    return out


IP_OPTS = (0, O.IP_CORNER, O.IP_BC_DIRICHLET, O.IP_BC_DIRICHLET_OLD, O.IP_CORNER | O.IP_BC_DIRICHLET,
           O.IP_RENDER_DENS)


def interp_points(n: int, res: int, bsx: int, seed: int) -> np.ndarray:
    """Points for the interpolation cases: uniform over the domain and 1.5 voxels beyond
    it, a quarter snapped to integers, half-integers and block upper faces."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = rng.uniform(-1.5, res + 1.5, (n, 3)).astype(np.float32)
    q = n // 4
    p[:q] = np.floor(p[:q]) + rng.choice(np.array([0.0, 0.5, 0.25], np.float32), (q, 3))
    p[q:2 * q, 0] = (rng.integers(0, res // bsx, q) * bsx + bsx - 0.5 +
                     rng.uniform(0, 1, q)).astype(np.float32)
    return p


def make_interp(small: dict) -> None:
    """Reference values of interpolateFloatFast / interpolateUint16ToFloatFast /
    interpolateRenderDensity (oracle/ref_driver.cpp, interp job)."""
    out = {}
    # (1) the golden MCF fields at the golden points (the particles of the surface)
    bids = small["active_bids"]
    for name, chan, key in (("f32", O.CHAN_F32, "pde_mcf8_f32"), ("u16", O.CHAN_U16, "pde_mcf8_u16_odd")):
        for opt in (0, O.IP_RENDER_DENS) if chan == O.CHAN_U16 else (0,):
            v, _, _ = O.run_reference_interp(RES, RES, RES, BSX, chan, bids, small[key], small["points"], opt)
            out[f"surf_{name}_{opt}"] = v
    # (2) a seeded payload on a layout that touches every face of a 32^3 domain, bs 8
    res, bs = 32, 8
    nb = (res // bs) ** 3
    rng = np.random.Generator(np.random.PCG64(20261203 + 920))
    rbids = np.nonzero(rng.random(nb) < 0.8)[0].astype(np.int32)
    u16 = rng.integers(0, 65536, (len(rbids), bs ** 3), dtype=np.uint16)
    f32 = (u16.astype(np.float32) * np.float32(1.0 / 65536.0)).astype(np.float32)
    pts = interp_points(2000, res, bs, 20261203 + 921)
    out.update(rand_res=np.int32(res), rand_bsx=np.int32(bs), rand_bids=rbids, rand_u16=u16, rand_points=pts)
    for name, chan, pay in (("f32", O.CHAN_F32, f32), ("u16", O.CHAN_U16, u16)):
        for opt in IP_OPTS:
            if chan == O.CHAN_F32 and opt & O.IP_RENDER_DENS:
                continue
            v, _, _ = O.run_reference_interp(res, res, res, bs, chan, rbids, pay, pts, opt)
            out[f"rand_{name}_{opt}"] = v
    path = os.path.join(HERE, "reference_interp.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


HALO_NB, HALO_BSX, HALO_LEVELS = (5, 4, 6), 8, 3
HALO_OPTS = (0, O.BC_NEUMANN, O.BC_COARSE_LEVEL)


def make_halo() -> None:
    """HaloBlockSet::fillHaloBlock_ of every block of each level of a 3-level channel
    (oracle/ref_driver.cpp, halo job): FP32 and uint16, options none / OPT_BC_NEUMANN /
    OPT_BC_COARSE_LEVEL, halo sizes 1 and 2."""
    import halo_cases as H
    import port as P
    out = {"nb": np.array(HALO_NB, np.int32), "bsx": np.int32(HALO_BSX), "n_levels": np.int32(HALO_LEVELS),
           "empty_value": np.float32(0.25), "full_value": np.float32(0.75)}
    res = [x * HALO_BSX for x in HALO_NB]
    for kind, chan in (("f32", O.CHAN_F32), ("u16", O.CHAN_U16)):
        lv, st, pay = H.halo_case(HALO_NB, HALO_BSX, HALO_LEVELS, 20261203 + 930 + chan, kind,
                                  lambda *a: P.regularize(*a)[0])
        out[f"{kind}_levels"] = lv
        for l in range(HALO_LEVELS):
            out[f"{kind}_state{l}"] = st[l]
            out[f"{kind}_pay{l}"] = pay[l]
        for L in range(HALO_LEVELS):
            for opt in HALO_OPTS:
                for h in (1, 2):
                    bids, vals = O.run_reference_halo(*res, HALO_BSX, HALO_LEVELS, chan, lv, st, pay, L, h, opt,
                                                      0.25, 0.75)
                    assert np.array_equal(bids, H.blocks_at(lv, st, L))
                    out[f"{kind}_L{L}_o{opt}_h{h}"] = vals
    path = os.path.join(HERE, "reference_halo.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


RENDER_CAMERAS = {
    "demo": dict(O.DEMO_CAMERA),
    "close": {"pos": (0.2, 0.55, 0.15), "look_at": (0.45, 0.45, 0.5), "sun": (-2.0, 3.0, -1.0),
              "color": (1.0, 1.0, 1.0), "zoom": 1.7},
}
RENDER_SIZES = ((160, 90), (320, 180))


def make_render(small: dict) -> None:
    """RDR::RaymarchRenderer::render (oracle/ref_driver.cpp, render job) of the golden uint16
    MCF field for two cameras and two image sizes: BMP_MKRGB pixels."""
    out = {}
    bids, pay = small["active_bids"], small["pde_mcf8_u16_odd"]
    for name, cam in RENDER_CAMERAS.items():
        for w, h in RENDER_SIZES:
            px, _, _ = O.run_reference_render(RES, RES, RES, BSX, bids, pay, w, h, cam)
            out[f"{name}_{w}x{h}"] = px
    path = os.path.join(HERE, "reference_render.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


MORTON_GRIDS = ((8, 8, 8), (13, 6, 10), (32, 32, 32), (40, 3, 17))


def make_morton() -> None:
    """MultiresSparseGrid::sortBlockListMorton (oracle/ref_driver.cpp, morton job) of seeded
    random lists (a third of each block grid, in random order) on 16^3 blocks."""
    out = {}
    rng = np.random.Generator(np.random.PCG64(20261203 + 940))
    for nb in MORTON_GRIDS:
        n = int(np.prod(nb))
        bids = rng.permutation(n)[: max(2, n // 3)].astype(np.int32)
        key = "x".join(map(str, nb))
        out[f"in_{key}"] = bids
        out[f"out_{key}"] = O.run_reference_morton(nb[0] * 16, nb[1] * 16, nb[2] * 16, 16, bids)
    path = os.path.join(HERE, "reference_morton.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def make_solver() -> None:
    """The reference's multiplyLaplacianMatrixOpt (Y = A X with sum(Y X), and B - A X),
    dotProdChannel, AXPBYChannelCombined and relax (relaxBlockList passes) on the seeded cases
    of tests/solver_cases.py (oracle/ref_driver.cpp, solver job)."""
    import port as P
    import solver_cases as S
    out = {}
    for name, res, bs, nblk, seed in S.SOLVER_CASES:
        bids, nb, prob, (x, b, q, p) = S.solver_case(P, res, bs, nblk, seed)
        coef = [prob.payload(v).astype(np.float32) for v in (prob.cx, prob.cy, prob.cz, prob.d)]
        for k, (passes, rev) in enumerate(S.RELAX_RUNS):
            r = O.run_reference_solver(res, res, res, bs, bids, x, b, q, p, *coef, a=S.AXPBY_A, bcoef=S.AXPBY_B,
                                       relax_passes=passes, reverse=rev)
            if k == 0:
                for key in ("ax", "residual", "axpby_x", "axpby_p"):
                    out[f"{name}_{key}"] = r[key]
                out[f"{name}_dots"] = np.array([r["dot_ax_x"], r["dot_x_b"]])
            out[f"{name}_relaxed_{passes}_{int(rev)}"] = r["relaxed"]
    path = os.path.join(HERE, "reference_solver.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def make_downsample() -> None:
    """downsampleFloatChannelNew to multigrid level 1 (oracle/ref_driver.cpp, downsample job)
    of seeded 3-level FP32 channels, 4^3 Gauss-like weights and OPT_SIMPLE_AVERAGE."""
    import halo_cases as H
    import port as P
    out = {}
    for nb, bsx, seed in H.DOWNSAMPLE_CASES:
        lv, st, pay = H.halo_case(nb, bsx, 3, seed, "f32", lambda *a: P.regularize(*a)[0])
        key = "x".join(map(str, nb)) + f"_bs{bsx}"
        for simple in (False, True):
            bids, vals = O.run_reference_downsample(*(n * bsx for n in nb), bsx, 3, lv, st, pay, simple,
                                                    H.DOWNSAMPLE_EMPTY, H.DOWNSAMPLE_FULL)
            out[f"{key}_bids"] = bids
            out[f"{key}_{'mean' if simple else 'gauss'}"] = vals
    path = os.path.join(HERE, "reference_downsample.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


SURFACE512_SAMPLE = 60000


def make_multires() -> None:
    """multiplyLaplacianMatrixOpt and relaxBlockList on multi-resolution layouts
    (oracle/ref_driver.cpp, multires job): Y = A X with sum(Y X), B - A X and the relaxed X
    for the seeded cases of tests/halo_cases.py, whose neighbouring levels meet through
    procNeighMixedRes2."""
    import halo_cases as H
    import port as P
    out = {}
    for nb, bsx, seed in H.MULTIRES_CASES:
        lv, x, b, dinv = H.multires_case(nb, bsx, 3, seed, lambda *a: P.regularize(*a)[0])
        key = "x".join(map(str, nb)) + f"_bs{bsx}"
        r = O.run_reference_multires(*(n * bsx for n in nb), bsx, 3, lv, x, b, dinv)
        out[f"{key}_levels"] = lv
        out[f"{key}_y"] = r["y"]
        out[f"{key}_r"] = r["r"]
        out[f"{key}_dot"] = np.float64(r["dot"])
        for passes, rev in H.MULTIRES_RELAX_RUNS:
            rr = O.run_reference_multires(*(n * bsx for n in nb), bsx, 3, lv, x, b, dinv, relax_passes=passes,
                                          reverse=rev)
            out[f"{key}_relaxed_{passes}_{int(rev)}"] = rr["relaxed"]
    path = os.path.join(HERE, "reference_multires.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def make_dense() -> None:
    """multiplyLaplacianMatrixOpt and relax() at the first dense multigrid level
    (oracle/ref_driver.cpp, dense job): Y = A X, B - A X and X after the Jacobi iterations for
    the seeded cases of tests/halo_cases.py."""
    import halo_cases as H
    out = {}
    for sx0, sy0, sz0, bsx, nl, seed in H.DENSE_CASES:
        key = f"{sx0}x{sy0}x{sz0}_L{nl}"
        case = H.dense_case(sx0, sy0, sz0, nl, seed)
        r = O.run_reference_dense(sx0, sy0, sz0, bsx, nl, *case)
        out[f"{key}_y"] = r["y"]
        out[f"{key}_r"] = r["r"]
        for it in H.DENSE_RELAX_ITERS:
            out[f"{key}_relaxed_{it}"] = O.run_reference_dense(sx0, sy0, sz0, bsx, nl, *case, relax_iter=it)["relaxed"]
    path = os.path.join(HERE, "reference_dense.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def make_layout() -> None:
    """setRefinementMap's block lists and CH_DIST_FINECOARSE (oracle/ref_driver.cpp, layout
    job) on the 3- and 4-level maps of reference_small.npz."""
    small = dict(np.load(os.path.join(HERE, "reference_small.npz")))
    out = {}
    for nl in (3, 4):
        r = O.run_reference_layout(8 * BSX, 8 * BSX, 8 * BSX, BSX, nl, small[f"lvl{nl}_in"])
        out[f"lvl{nl}_existing"] = r["existing"]
        for l in range(nl):
            out[f"lvl{nl}_fine_coarse{l}"] = r["fine_coarse"][l]
            d = r["dist"][l]
            out[f"lvl{nl}_dist{l}_value_bids"] = d["value_bids"]
            out[f"lvl{nl}_dist{l}_value"] = d["value"]
            out[f"lvl{nl}_dist{l}_full_bids"] = d["full_bids"]
            out[f"lvl{nl}_dist{l}_full_value"] = np.uint16(d["full_value"])
    path = os.path.join(HERE, "reference_layout.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def make_halo3() -> None:
    """HaloBlockSet::fillHaloBlock3 at multigrid level 0 (oracle/ref_driver.cpp, halo3 job) of
    every level-0 block of seeded 3-level FP32 channels with seeded cell flags, for the domain
    boundary types of tests/halo_cases.py."""
    import halo_cases as H
    import port as P
    out = {}
    for nb, bsx, seed, dbc in H.HALO3_CASES:
        lv, st, pay = H.halo_case(nb, bsx, 3, seed, "f32", lambda *a: P.regularize(*a)[0])
        fst, fpay, ef, ff = H.flags_case(st, bsx, seed + 100)
        key = "x".join(map(str, nb)) + f"_bs{bsx}"
        bids, vals = O.run_reference_halo3(*(n * bsx for n in nb), bsx, 3, lv, st, pay, fst, fpay, dbc,
                                           H.DOWNSAMPLE_EMPTY, H.DOWNSAMPLE_FULL, ef, ff)
        out[f"{key}_bids"] = bids
        out[f"{key}_halo"] = vals
    path = os.path.join(HERE, "reference_halo3.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def make_surface512() -> None:
    """The 512^3 surface workload at full size (64 spheres x 32,000 points, bs 16, 20 MCF
    iterations, dt 0.1) through the reference, FP32 and uint16: active blocks, levels, flags,
    particle counts, per-block sums of the finalized and swept fields, and a seeded sample of
    their voxels (the full fields are 50 MB each)."""
    from msbg_gb300 import workloads as W
    spec = W.SURFACE_512
    pts = W.make_points(spec, 1)
    res, bsx = spec["res"], spec["bsx"]
    out = {}
    for name, chan in (("f32", O.CHAN_F32), ("u16", O.CHAN_U16)):
        r = O.run_reference_surface(O.SurfaceJob(res, res, res, bsx, pts, chan=chan, n_iter=spec["n_iter"],
                                                 dt=spec["dt"]), timeout=3600)
        if "active_bids" not in out:
            out.update(active_bids=r.active_bids, levels=r.levels, flags=r.flags,
                       n_act_particles=np.int64(r.n_act_particles))
            rng = np.random.Generator(np.random.PCG64(20261203 + 970))
            out["sample_index"] = np.sort(rng.choice(r.after_pde.size, SURFACE512_SAMPLE, replace=False))
        else:
            assert np.array_equal(out["active_bids"], r.active_bids)
        idx = out["sample_index"]
        for stage, field in (("final", r.after_finalize), ("pde", r.after_pde)):
            out[f"{name}_{stage}_block_sums"] = field.astype(np.float64).sum(axis=1)
            out[f"{name}_{stage}_sample"] = field.reshape(-1)[idx]
    path = os.path.join(HERE, "reference_surface512.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main(sys.argv[1:])
