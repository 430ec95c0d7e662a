"""Seeded batch of independent sparse Poisson volumes (the batched-solve workload).

256 volumes, each a union of 1 to 40 seeded spheres in its own 1024^3 domain with
base block 16^3 (64^3 blocks per volume).  A volume's target active-block count is
lognormal (median ``median_blocks``, sigma ``sigma``) clipped to [50, 20,000]; its
sphere radii are scaled so that the spheres' shells of blocks reach about that
count (a block is active when it lies within 4 voxels of a sphere surface, the
splat's marking radius).  The volumes are laid out in an 8 x 8 x 4 super-grid of
64^3-block cells of one block grid (8192 x 8192 x 4096 voxels); the sphere
centres keep every active block at least 4 blocks inside its cell, so volumes
never share a block face and the multigrid aggregation (2x2x2 per level) keeps
them apart down to one cell per volume.
"""
from __future__ import annotations

import numpy as np

from . import workloads as W

VOL_BLOCKS = 64          # block edge of one volume's domain
SUPER = (8, 8, 4)        # volumes along x, y, z
BS = 16


def volume_spheres(v: int, median_blocks: float = 600.0, sigma: float = 1.2):
    """Seeded spheres (centres, radii in voxels of the volume's own domain) and the
    target block count of volume v."""
    rng = np.random.Generator(np.random.PCG64(W.workload_seed(5, v)))
    target = float(np.clip(rng.lognormal(np.log(median_blocks), sigma), 50, 20000))
    k = int(rng.integers(1, 41))
    u = rng.uniform(0.5, 1.0, k)
    # blocks of a shell of radius r (voxels): ~ 4 pi r^2 * (2*(13.9+4)) / 16^3
    per_r2 = 4 * np.pi * 2 * (BS * np.sqrt(3) / 2 + 4) / BS ** 3
    R = np.sqrt(target / (per_r2 * np.sum(u * u)))
    r = np.clip(R * u, 2.0, 0.3 * VOL_BLOCKS * BS)
    lo = 4 * BS + r
    hi = (VOL_BLOCKS - 4) * BS - r
    c = rng.uniform(0, 1, (k, 3)) * (hi - lo)[:, None] + lo[:, None]
    return c, r, target


def volume_blocks(c: np.ndarray, r: np.ndarray) -> np.ndarray:
    """Active-block mask [64,64,64] (z, y, x) of one volume: blocks whose centre lies
    within 4 voxels + half a block diagonal of a sphere surface."""
    m = np.zeros((VOL_BLOCKS,) * 3, bool)
    h = BS * np.sqrt(3) / 2 + 4.0
    for ci, ri in zip(c, r):
        lo = np.maximum(((ci - ri - h) // BS).astype(int), 0)
        hi = np.minimum(((ci + ri + h) // BS).astype(int) + 1, VOL_BLOCKS)
        zz, yy, xx = np.meshgrid(np.arange(lo[2], hi[2]), np.arange(lo[1], hi[1]), np.arange(lo[0], hi[0]),
                                 indexing="ij")
        d = np.sqrt((xx * BS + BS / 2 - ci[0]) ** 2 + (yy * BS + BS / 2 - ci[1]) ** 2 + (zz * BS + BS / 2 - ci[2]) ** 2)
        m[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] |= np.abs(d - ri) <= h
    return m


def batch_layout(n_vol: int = 256, median_blocks: float = 600.0, sigma: float = 1.2):
    """Level map (int32, 0 = value block, 1 = empty) and volume of every block of the
    combined grid; grid size in voxels; per-volume target counts."""
    sx, sy, sz = SUPER
    nbx, nby, nbz = sx * VOL_BLOCKS, sy * VOL_BLOCKS, sz * VOL_BLOCKS
    levels = np.ones((nbz, nby, nbx), np.int32)
    vol = np.full((nbz, nby, nbx), -1, np.int32)
    targets = []
    for v in range(n_vol):
        vx, vy, vz = v % sx, (v // sx) % sy, v // (sx * sy)
        c, r, target = volume_spheres(v, median_blocks, sigma)
        targets.append(target)
        m = volume_blocks(c, r)
        sl = (slice(vz * VOL_BLOCKS, (vz + 1) * VOL_BLOCKS), slice(vy * VOL_BLOCKS, (vy + 1) * VOL_BLOCKS),
              slice(vx * VOL_BLOCKS, (vx + 1) * VOL_BLOCKS))
        levels[sl][m] = 0
        vol[sl][m] = v
    return levels.reshape(-1), vol.reshape(-1), (nbx * BS, nby * BS, nbz * BS), np.asarray(targets)


def run_batch(steps: int = 3, warmup: int = 1, learned_weights: str | None = None, n_vol: int = 256,
              tol: float = 1e-6) -> dict:
    """Builds the batch, solves it with the segmented MG-PCG (CUDA graph per
    iteration) from X = 0 -- and, with ``learned_weights``, from the learned warm
    start -- and reports solves/s and per-volume times to tolerance."""
    from . import gpu as G
    from . import poisson_workload as PW

    levels, vol, dims, targets = batch_layout(n_vol)
    g = G.MultiresSparseGrid(dims[0], dims[1], dims[2], BS, 2, G.F16)
    try:
        g.set_levels(levels)
        g.setRefinementMap(0.0)
        for ch in (PW.CH_X, PW.CH_B):
            g.channel_create(ch, G.F32)
        g.poisson_procedural_coefficients(PW.COEFF_SEED)
        bids = g.active_blocks().astype(np.int64)
        nb = (g.nbx, g.nby, g.nbz)
        b = PW.seeded_rhs(bids, nb, BS, 5000)
        g.upload_payload(b, PW.CH_B)
        del b
        g.batch_set_volumes(vol, n_vol)
        blocks = np.bincount(vol[vol >= 0], minlength=n_vol)
        out = {"workload": f"poisson-batch{n_vol}-1024^3-bs16", "volumes": n_vol, "cells": int(len(bids)) * BS ** 3,
               "blocks_per_volume": {"min": int(blocks.min()), "p50": float(np.median(blocks)),
                                     "p99": float(np.percentile(blocks, 99)), "max": int(blocks.max())},
               "tolerance": tol}

        def one(kind, use_graph=True):
            g.synchronize()
            ms_pred = 0.0
            if kind == "learned":
                g.event_record(2)
                g.warmnet_predict(PW.CH_B, PW.CH_X)
                g.event_record(3)
                g.synchronize()
                ms_pred = g.event_elapsed_ms(2, 3)
            else:
                g.fill(0.0, PW.CH_X)
                g.synchronize()
            its, ms, rel, tot = g.batch_mgpcg_solve(PW.CH_X, PW.CH_B, tol=tol, max_iter=100, use_graph=use_graph)
            return its, ms + ms_pred, rel, tot + ms_pred

        kinds = [("plain", True), ("plain_no_graph", False)]
        if learned_weights:
            W_, c_ = PW.load_warmnet(learned_weights)
            g.warmnet_set(W_, c_)
            kinds.append(("learned", True))
        for name, use_graph in kinds:
            kind = "learned" if name == "learned" else "plain"
            for _ in range(warmup):
                one(kind, use_graph)
            runs = [one(kind, use_graph) for _ in range(steps)]
            its, ms, rel, tot = sorted(runs, key=lambda r: r[3])[len(runs) // 2]
            ok = its >= 0
            out[name] = {"batch_ms": tot, "solves_per_s": n_vol / (tot / 1e3),
                         "per_volume_ms_p50": float(np.percentile(ms[ok], 50)) if ok.any() else None,
                         "per_volume_ms_p99": float(np.percentile(ms[ok], 99)) if ok.any() else None,
                         "iterations_mean": float(its[ok].mean()) if ok.any() else None,
                         "iterations_max": int(its.max()), "converged": int(ok.sum()),
                         "max_rel_residual_fp64": float(rel.max())}
        # the operator launch shapes the autotuner picked for the batch's levels (level,
        # bytes per value, mode, cells per thread, grid)
        out["operator_shapes"] = [list(t) for t in g.poisson_tuning()]
        return out
    finally:
        g.close()
