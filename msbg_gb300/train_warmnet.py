"""Trains the learned warm start of the Poisson solve on the GPU.

Training family: the Poisson problem of poisson_workload on the level-0 blocks of
the first ``--clusters`` clusters of the 4096^3 layout (seeded coefficients), with
right-hand sides from seeds 1..N (N = ``--pairs``, 2,000 by default).  For every
seed the plain FP32 MG-PCG produces the solution x* (relative residual 1e-6);
the pairs stay in device memory.  The network (msbg_gpu_warmnet_*) trains with
Adam on the loss ||x1 - avg(x*)||^2 / ||avg(x*)||^2 (level-1 value against the
mean of its level-0 children of x*; ``--loss residual``: ||A (x0 - x*)||^2 / ||b||^2),
one pair per step.  Evaluation:
``--eval`` held-out seeds (10,001 upward) are solved from X = 0 and from the
network's starting point; iterations, wall time and the initial relative residual
are reported.

    python -m msbg_gb300.train_warmnet --out msbg_gb300/data/warmnet_c3.npz
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from msbg_gb300 import gpu as G  # noqa: E402
from msbg_gb300 import poisson_workload as PW  # noqa: E402

CH = (2, 16, 16, 16, 2)


def init_weights(seed: int):
    """He-normal weights (last layer scaled by 1/2), zero biases."""
    rng = np.random.Generator(np.random.PCG64(seed))
    W, c = [], []
    for l in range(4):
        cin, cout = CH[l], CH[l + 1]
        std = np.sqrt(2.0 / (27 * cin)) * (0.5 if l == 3 else 1.0)
        W.append(rng.normal(0.0, std, (27, cin, cout)).astype(np.float32))
        c.append(np.zeros(cout, np.float32))
    return W, c


def coarse_average(x: np.ndarray, bs: int) -> np.ndarray:
    """Every level-0 value replaced by the mean of its 2x2x2 group (payload layout)."""
    h = bs // 2
    a = x.reshape(-1, h, 2, h, 2, h, 2).mean(axis=(2, 4, 6), keepdims=True)
    return np.broadcast_to(a, (x.shape[0], h, 2, h, 2, h, 2)).reshape(x.shape).astype(np.float32)


def evaluate(g, bids, nb, bs, labels, seeds, tol=1e-6, ideal: int = 20) -> dict:
    """Held-out seeds solved from X = 0 and from the network's start; for the first
    `ideal` seeds also from the best coarse start (the solution's own 2x2x2 means)."""
    n0 = len(bids) * bs ** 3
    its_zero, its_warm, ms_zero, ms_warm, its_ideal = [], [], [], [], []
    for k, sd in enumerate(seeds):
        b = PW.seeded_rhs(bids, nb, bs, sd, labels)
        g.upload_payload(b, PW.CH_B)
        r = PW.timed_solve(g, "plain", tol=tol)
        its_zero.append(r["iterations"]); ms_zero.append(r["ms"])
        if k < ideal:
            g.mgpcg_solve(PW.CH_X, PW.CH_B, tol=3e-7, max_iter=200)
            g.upload_payload(coarse_average(g.payload(PW.CH_X), bs), PW.CH_X)
            its_ideal.append(g.mgpcg_solve(PW.CH_X, PW.CH_B, tol=tol, max_iter=200)[0])
        r = PW.timed_solve(g, "learned", tol=tol)
        its_warm.append(r["iterations"]); ms_warm.append(r["ms"])
    return {"seeds": len(seeds), "iterations_zero_mean": float(np.mean(its_zero)),
            "iterations_learned_mean": float(np.mean(its_warm)),
            "iterations_ideal_coarse_start_mean": float(np.mean(its_ideal)) if its_ideal else None,
            "ms_zero_median": float(np.median(ms_zero)), "ms_learned_median": float(np.median(ms_warm)),
            "cells": int(n0)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--clusters", type=int, default=1)
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--eval", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--loss", default="coarse", choices=["coarse", "residual"])
    ap.add_argument("--load", default=None, help="evaluate these weights (npz) instead of training")
    ap.add_argument("--out", default=os.path.join(ROOT, "msbg_gb300", "data", "warmnet_c3.npz"))
    args = ap.parse_args()

    t0 = time.time()
    g, spec = PW.surface_layout_grid(args.clusters)
    bs = spec["bsx"]
    bids, _ = PW.setup_problem(g, bs)
    nb = (g.nbx, g.nby, g.nbz)
    labels = PW.component_labels(bids, nb)
    n0 = len(bids) * bs ** 3
    W, c = init_weights(args.seed) if args.load is None else PW.load_warmnet(args.load)
    g.warmnet_set(W, c)
    g.warmnet_set_loss(args.loss)
    if args.load is not None:
        ev = evaluate(g, bids, nb, bs, labels, range(10001, 10001 + args.eval))
        g.close()
        print(json.dumps({"weights": args.load, "cells": int(n0), "eval": ev}), flush=True)
        return

    # (b, x*) pairs from the plain solver, kept in device memory
    slab = G.DeviceBuffer.alloc(2 * args.pairs * n0 * 4)
    t_gen = time.time()
    for k in range(args.pairs):
        b = PW.seeded_rhs(bids, nb, bs, 1 + k, labels)
        g.upload_payload(b, PW.CH_B)
        g.fill(0.0, PW.CH_X)
        it, rel = g.mgpcg_solve(PW.CH_X, PW.CH_B, tol=1e-6, max_iter=200)
        g.copy_d2d(slab.ptr + (2 * k) * n0 * 4, g.payload_ptr(PW.CH_B), n0 * 4)
        g.copy_d2d(slab.ptr + (2 * k + 1) * n0 * 4, g.payload_ptr(PW.CH_X), n0 * 4)
    g.synchronize()
    t_gen = time.time() - t_gen

    rng = np.random.default_rng(args.seed)
    t_train = time.time()
    history = []
    step = 0
    total = args.epochs * args.pairs
    for ep in range(args.epochs):
        order = rng.permutation(args.pairs)
        losses = []
        for k in order:
            lr = args.lr * 0.5 * (1.0 + np.cos(np.pi * step / total))  # cosine decay
            losses.append(g.warmnet_train_step(slab.ptr + (2 * k) * n0 * 4, slab.ptr + (2 * k + 1) * n0 * 4, lr))
            step += 1
        history.append(float(np.mean(losses)))
        print(f"epoch {ep}: mean loss {history[-1]:.5f}", flush=True)
    g.synchronize()
    t_train = time.time() - t_train
    slab.free()

    W, c = g.warmnet_get()
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    np.savez(args.out, **{f"W{l}": W[l] for l in range(4)}, **{f"c{l}": c[l] for l in range(4)})
    ev = evaluate(g, bids, nb, bs, labels, range(10001, 10001 + args.eval))
    g.close()
    summary = {"clusters": args.clusters, "cells": int(n0), "pairs": args.pairs, "epochs": args.epochs,
               "loss_per_epoch": history, "generate_s": t_gen, "train_s": t_train, "eval": ev,
               "total_s": time.time() - t0, "weights": os.path.relpath(args.out, ROOT)}
    print(json.dumps(summary), flush=True)


if __name__ == "__main__":
    main()
