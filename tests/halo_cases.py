"""Seeded multi-level channel layouts for the cross-resolution halo fill tests.

A case is a regular level map (levels grow with the distance from one corner of the block
grid, with seeded jitter, then regularizeRefinementMap) and, for every resolution level
l, per-block states and a payload of (bsx>>l)^3 values per payload block:
  - blocks at level l: a payload block, now and then the constant empty or full block;
  - other blocks: a payload block (ghost data), the constant empty block or no block;
  - the coarsest level has a block everywhere, and a block without a block at level l
    has one at level l+1, so every coarse-level read of the halo fill finds data, as the
    reference requires (src/halo.h:310-322).
Payload values: uint16 uniform; FP32 the uint16 values / 65536; FP16 the FP32 values
rounded to half.
"""
from __future__ import annotations

import numpy as np

LBLK_EMPTY, LBLK_FULL, LBLK_NONE = -1, -2, -3

# restriction fixtures (downsampleFloatChannelNew): (block grid, block edge, seed), and the
# constant blocks' values
DOWNSAMPLE_CASES = (((4, 4, 4), 16, 20261203 + 960), ((5, 3, 4), 8, 20261203 + 961),
                    ((3, 3, 2), 32, 20261203 + 962))
DOWNSAMPLE_EMPTY, DOWNSAMPLE_FULL = 0.25, 0.75
# the solver's halo (fillHaloBlock3): (block grid, block edge, seed, domain boundary types of
# faces -x,+x,-y,+y,-z,+z; 0 open, 1 solid)
HALO3_CASES = (((4, 4, 4), 16, 20261203 + 980, (0, 1, 0, 1, 1, 0)),
               ((5, 3, 4), 8, 20261203 + 981, (1, 1, 0, 0, 1, 0)))


def halo_case(nb, bsx: int, n_levels: int, seed: int, kind: str, regularize):
    """kind: 'f32' | 'u16' | 'f16'; regularize(levels, nbx, nby, nbz, n_levels) -> levels."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = int(np.prod(nb))
    bz, by, bx = np.meshgrid(np.arange(nb[2]), np.arange(nb[1]), np.arange(nb[0]), indexing="ij")
    d = (bx + by + bz).ravel() + rng.integers(-1, 2, n)
    lv = np.clip(d // 3, 0, n_levels - 1).astype(np.int32)
    lv = np.asarray(regularize(lv, nb[0], nb[1], nb[2], n_levels), np.int32)
    states, pays = [], []
    for l in range(n_levels):
        st = np.full(n, LBLK_NONE, np.int32)
        r = rng.random(n)
        own = lv == l
        st[~own & (r < 0.3)] = 0
        st[~own & (r >= 0.3) & (r < 0.4)] = LBLK_EMPTY
        st[own] = 0
        st[own & (r < 0.05)] = LBLK_EMPTY
        st[own & (r >= 0.05) & (r < 0.08)] = LBLK_FULL
        if l == n_levels - 1:
            st[st == LBLK_NONE] = 0
        states.append(st)
    for l in range(n_levels - 2, -1, -1):
        miss = (states[l] == LBLK_NONE) & (states[l + 1] == LBLK_NONE)
        states[l + 1][miss] = LBLK_EMPTY
    for l in range(n_levels):
        st = states[l]
        k = st == 0
        st[k] = np.arange(int(k.sum()), dtype=np.int32)
        bs = bsx >> l
        u16 = rng.integers(0, 65536, (int(k.sum()), bs ** 3)).astype(np.uint16)
        if kind == "u16":
            pays.append(u16)
        else:
            f32 = (u16.astype(np.float32) * np.float32(1.0 / 65536.0)).astype(np.float32)
            pays.append(f32 if kind == "f32" else f32.astype(np.float16))
    return lv, states, pays


def blocks_at(lv, states, level):
    """Blocks whose level is `level` and that have a block at that level, ascending."""
    return np.nonzero((np.asarray(lv) == level) & (states[level] != LBLK_NONE))[0].astype(np.int32)


# cell flags (src/msbg.h:602-614): the two the solver's halo reads, and others it ignores
CELL_SOLID, CELL_PARTIAL_SOLID, CELL_VOID, CELL_AIR = 1 << 0, 1 << 6, 1 << 12, 1 << 2


def flags_case(states, bsx: int, seed: int):
    """Cell flags for the levels of a halo case: the same block states as the values, each
    payload cell CELL_VOID (8 %), CELL_SOLID (8 %) or other bits; constant blocks' flags."""
    rng = np.random.Generator(np.random.PCG64(seed))
    fpay = []
    for l, st in enumerate(states):
        n = int(st.max()) + 1 if len(st) and st.max() >= 0 else 0
        u = rng.random((n, (bsx >> l) ** 3))
        f = np.where(u < 0.08, CELL_VOID, np.where(u < 0.16, CELL_SOLID, np.where(u < 0.5, CELL_PARTIAL_SOLID,
                                                                                     CELL_AIR)))
        fpay.append(f.astype(np.uint16))
    return [s.copy() for s in states], fpay, CELL_VOID | CELL_AIR, CELL_AIR


# the solver operator on multi-resolution layouts (multiplyLaplacianMatrixOpt with
# procNeighMixedRes2): (block grid, block edge, seed).  The reference's operator takes block
# edges 16, 8, 4 and 2 (an edge-32 layout stops it with an assertion).
MULTIRES_CASES = (((4, 4, 4), 16, 20261203 + 990), ((5, 3, 4), 8, 20261203 + 991),
                  ((6, 5, 4), 16, 20261203 + 992))
# relaxBlockList runs on them: (passes, reverse order)
MULTIRES_RELAX_RUNS = ((1, False), (2, True))


def multires_case(nb, bsx: int, n_levels: int, seed: int, regularize):
    """A regular level map (as halo_case) with every block a fluid block at its level, and
    float32 X, B and the diagonal channel's values over the blocks of level 0, then level 1,
    ..., ascending bid: X, B standard normal, the diagonal uniform in [0.1, 0.2] with about
    1% zeros (cells the operator sets to 0).  Returns (levels, x, b, dinv)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = int(np.prod(nb))
    bz, by, bx = np.meshgrid(np.arange(nb[2]), np.arange(nb[1]), np.arange(nb[0]), indexing="ij")
    d = (bx + by + bz).ravel() + rng.integers(-1, 2, n)
    lv = np.clip(d // 2, 0, n_levels - 1).astype(np.int32)
    lv = np.asarray(regularize(lv, nb[0], nb[1], nb[2], n_levels), np.int32)
    total = sum(int((lv == l).sum()) * (bsx >> l) ** 3 for l in range(n_levels))
    x = rng.standard_normal(total).astype(np.float32)
    b = rng.standard_normal(total).astype(np.float32)
    dinv = rng.uniform(0.1, 0.2, total).astype(np.float32)
    dinv[rng.random(total) < 0.01] = 0.0
    return lv, x, b, dinv


# the solver operator at the first dense multigrid level: (domain sx, sy, sz of level 0,
# block edge, resolution levels (the dense level is levelMg = this), seed)
DENSE_CASES = ((80, 96, 64, 16, 2, 20261203 + 1000), (80, 96, 64, 16, 3, 20261203 + 1001),
               (112, 48, 80, 16, 2, 20261203 + 1002))
CELL_SOLID, CELL_PARTIAL_SOLID, CELL_VOID = 1 << 0, 1 << 6, 1 << 12
# relax() iteration counts run at that level (odd: the result is copied back from the
# temporary channel)
DENSE_RELAX_ITERS = (1, 4)


def dense_case(sx0, sy0, sz0, n_levels, seed):
    """Arrays [sz][sy][sx] of the dense level levelMg = n_levels (edges sx0 >> n_levels, ...):
    cell flags (10% solid, 10% void, 15% partially solid, the rest fluid), X and B standard
    normal, the diagonal channel uniform in [0.1, 0.2] with about 2% zeros, face areas uniform
    in [0.3, 1]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = (sz0 >> n_levels, sy0 >> n_levels, sx0 >> n_levels)
    r = rng.random(s)
    flags = np.where(r < 0.1, CELL_SOLID, np.where(r < 0.2, CELL_VOID,
                                                   np.where(r < 0.35, CELL_PARTIAL_SOLID, 0))).astype(np.uint16)
    x = rng.standard_normal(s).astype(np.float32)
    b = rng.standard_normal(s).astype(np.float32)
    dinv = rng.uniform(0.1, 0.2, s).astype(np.float32)
    dinv[rng.random(s) < 0.02] = 0.0
    ax, ay, az = (rng.uniform(0.3, 1.0, s).astype(np.float32) for _ in range(3))
    return flags, x, b, dinv, ax, ay, az
