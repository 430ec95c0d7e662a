"""Seeded inputs for the solver building blocks (the reference's multiplyLaplacianMatrixOpt,
dotProdChannel, AXPBYChannelCombined and block smoother), shared by the fixture generator and
the tests: a random set of value blocks on a cubic grid, the seeded face coefficients of the
GPU's procedural set (restated by the oracle's PoissonProblem) and four random fields X, B, Q, P
as FP32 payloads [n][bs^3] in ascending block id."""
from __future__ import annotations

import numpy as np

# (name, grid edge, block edge, value blocks, seed)
SOLVER_CASES = (("bs16", 64, 16, 8, 20261203 + 950), ("bs8", 64, 8, 32, 20261203 + 951))
COEFF_SEED = 4242
AXPBY_A, AXPBY_B = 0.5, -2.0
# relax runs: (passes, reverse)
RELAX_RUNS = ((1, False), (2, True))


def solver_case(port, res: int, bs: int, n_blocks: int, seed: int):
    nb = (res // bs,) * 3
    rng = np.random.Generator(np.random.PCG64(seed))
    bids = np.sort(rng.choice(int(np.prod(nb)), n_blocks, replace=False)).astype(np.int32)
    prob = port.PoissonProblem(bids.astype(np.int64), nb, bs, seed=COEFF_SEED)
    fields = [rng.standard_normal((n_blocks, bs ** 3)).astype(np.float32) for _ in range(4)]
    return bids, nb, prob, fields
