"""Seeded sparse Poisson problems on the surface-reconstruction block layouts.

The Poisson workload uses the level-0 blocks of the 4096^3 three-level layout
(or of a crop of it: its first N clusters) as the set of unknowns:

* operator: 7-point, variable face coefficients uniform in [0.5, 2] from a seeded
  hash of the face position (``msbg_gpu_poisson_procedural_coefficients``),
  Dirichlet 0 outside the active blocks;
* right-hand side: N(0, 1) per active cell (numpy PCG64, seed
  ``workload_seed(3, index)``), projected to zero mean over every 6-connected
  component of active blocks (blocks sharing a face; all cells of an active
  block are active, so block connectivity is cell connectivity);
* tolerance: relative residual 1e-6 checked with the double-float residual and
  FP64 norms.
"""
from __future__ import annotations

import numpy as np

from . import gpu as G
from . import workloads as W

CH_X, CH_B = 1, 2
COEFF_SEED = 20264242


def component_labels(bids: np.ndarray, nb) -> tuple[np.ndarray, int]:
    """Label of every active block's 6-connected component (1-based) and their count."""
    from scipy import ndimage

    nbx, nby, nbz = nb
    mask = np.zeros(nbx * nby * nbz, np.uint8)
    mask[bids] = 1
    lab, n = ndimage.label(mask.reshape(nbz, nby, nbx))
    return lab.reshape(-1)[bids], int(n)


def seeded_rhs(bids: np.ndarray, nb, bs: int, index: int = 0, labels=None) -> np.ndarray:
    """RHS payload [nActive][bs^3] (float32): N(0,1), zero mean per component
    (``labels`` = component_labels(bids, nb), computed when not given)."""
    rng = np.random.Generator(np.random.PCG64(W.workload_seed(3, index)))
    b = rng.standard_normal((len(bids), bs ** 3), dtype=np.float32)
    blab, ncomp = labels if labels is not None else component_labels(bids, nb)
    sums = np.bincount(blab, weights=b.sum(axis=1, dtype=np.float64), minlength=ncomp + 1)
    cnt = np.bincount(blab, minlength=ncomp + 1).astype(np.float64) * bs ** 3
    mean = (sums / np.maximum(cnt, 1.0)).astype(np.float32)
    b -= mean[blab][:, None]
    return b


def surface_layout_grid(n_objects: int | None = None, workload_index: int = 2):
    """A context with the level-0 block layout of the 4096^3 surface workload (or of
    its first ``n_objects`` clusters); returns (grid, spec)."""
    spec = dict(W.SURFACE_4096)
    if n_objects is not None:
        spec["n_objects"] = n_objects
    pts = W.make_points(spec, workload_index)
    g = G.MultiresSparseGrid(spec["res"], spec["res"], spec["res"], spec["bsx"], spec["n_levels"], G.F16)
    d = g.to_device(pts)
    g.levels_from_bands(d, len(pts), (spec["fine_band"], spec["mid_band"]))
    g.regularizeRefinementMap()
    g.setRefinementMap(0.0)
    d.free()
    return g, spec


def setup_problem(g, bs: int, rhs_index: int = 0):
    """FP32 channels X, B, the seeded coefficients and RHS on grid g; returns the
    active block ids and the RHS payload."""
    for ch in (CH_X, CH_B):
        g.channel_create(ch, G.F32)
    g.poisson_procedural_coefficients(COEFF_SEED)
    bids = g.active_blocks().astype(np.int64)
    b = seeded_rhs(bids, (g.nbx, g.nby, g.nbz), bs, rhs_index)
    g.upload_payload(b, CH_B)
    return bids, b


def load_warmnet(path: str):
    """Trained warm-start weights (npz with W0..W3, c0..c3)."""
    z = np.load(path)
    return [z[f"W{l}"] for l in range(4)], [z[f"c{l}"] for l in range(4)]


def timed_solve(g, kind: str, tol: float = 1e-6, max_iter: int = 200, inner_tol: float = 3e-2,
                max_outer: int = 12, max_inner: int = 60) -> dict:
    """One solve, timed with CUDA events on the context's stream: from X = 0
    ("plain", "mixed") or from the learned warm start ("learned", "learned_mixed";
    the network's forward pass is inside the timed region).  The mixed solves stop
    each FP16 inner solve at a relative residual of inner_tol (3e-2: four outer
    steps of about two inner iterations; on the 4096^3 layout 1.45 s against 1.59 s
    with 3e-3 and 1.81 s with 1e-2); the outer loop still stops on the FP64-checked
    residual of the FP32 system."""
    g.synchronize()
    l0 = g.launch_count()
    if kind.startswith("learned"):
        g.event_record(0)
        g.warmnet_predict(CH_B, CH_X)
    else:
        g.fill(0.0, CH_X)
        g.event_record(0)
    if kind in ("plain", "learned"):
        it, rel = g.mgpcg_solve(CH_X, CH_B, tol=tol, max_iter=max_iter)
        extra = {"iterations": it}
    else:
        o, i, rel = g.mgpcg_solve_mixed(CH_X, CH_B, tol=tol, max_outer=max_outer, inner_tol=inner_tol,
                                        max_inner=max_inner)
        extra = {"outer_steps": o, "inner_iterations": i}
    g.event_record(1)
    g.synchronize()
    return {"ms": g.event_elapsed_ms(0, 1), "rel_residual": rel, "gpu_launches": g.launch_count() - l0, **extra}
