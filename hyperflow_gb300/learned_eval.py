"""Trains the learned coarse solver on fine FP64 runs of the plain solver and evaluates it.

    python -m hyperflow_gb300.learned_eval [--n-fine 2048] [--iters 3000] [--out report.json]

Training data: 4x box-filtered FP64 runs at n_fine of two seeded four-quadrant Riemann
problems and two shock-bubble flows (Mach 1.22 shock, bubble density 0.138, radius 0.2).
Evaluation on held-out cases (another Riemann seed, another bubble placement): L1 density
error against the filtered FP64 n_fine solution and wall time of
  * plain FP64 MUSCL-Hancock at n_fine (the reference itself), n_fine/2 and n_fine/4,
  * plain FP32 and learned FP32 at n_fine/4.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import cases
from .learned import LearnedSolver, evaluate, fine_pairs, init_params, one_step_loss, train


def sb_case(bubble, radius, t_end):
    return lambda n: cases.shock_bubble_case(n, bubble=bubble, radius=radius, t_end=t_end)


def rp_case(seed):
    return lambda n: cases.random_quadrant_case(n, seed)


def _log(msg: str, t0: float):
    print(f"[{time.perf_counter() - t0:8.1f} s] {msg}", file=sys.stderr, flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-fine", type=int, default=2048)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--stride", type=int, default=8)
    ap.add_argument("--out", default="learned_report.json")
    args = ap.parse_args()
    nf, f = args.n_fine, 4
    nc = nf // f
    report = {"n_fine": nf, "n_coarse": nc}
    t0 = time.perf_counter()
    train_sets = [("rp_seed_100", rp_case(100), None), ("rp_seed_101", rp_case(101), None),
                  ("bubble_a", sb_case((0.4, 0.5), 0.2, 1.0), 0.25),
                  ("bubble_b", sb_case((0.45, 0.45), 0.2, 1.0), 0.25)]
    pairs = []
    for name, fn, t_end in train_sets:
        c = fn(nf)
        T = t_end if t_end is not None else c["simulation"]["t_end"]
        pairs += fine_pairs(c, T, factor=f, stride=args.stride)
        _log(f"fine data {name}: {len(pairs)} pairs", t0)
    report["train_pairs"] = len(pairs)
    report["data_seconds"] = time.perf_counter() - t0
    held_pairs = fine_pairs(rp_case(200)(nf), rp_case(200)(nf)["simulation"]["t_end"], factor=f,
                            stride=args.stride * 2)
    held_pairs += fine_pairs(cases.shock_bubble_case(nf, bubble=(0.42, 0.55)), 0.2, factor=f,
                             stride=args.stride * 2)
    _log(f"held-out data: {len(held_pairs)} pairs", t0)
    ls = LearnedSolver(nc, 1.0 / nc)
    ls.set_params(init_params(0))
    t1 = time.perf_counter()
    losses, w = train(ls, pairs, args.iters, lr=args.lr)
    report["train_seconds"] = time.perf_counter() - t1
    _log(f"trained {args.iters} iterations in {report['train_seconds']:.1f} s", t0)
    report["train_loss_first100"] = float(losses[:100].mean())
    report["train_loss_last100"] = float(losses[-100:].mean())
    report["heldout_one_step_loss"] = {"plain": one_step_loss(ls, held_pairs, w, False),
                                       "learned": one_step_loss(ls, held_pairs, w, True)}
    params = ls.params()
    ls.close()
    np.save(args.out.replace(".json", "_params.npy"), params)
    report["eval"] = {}
    report["eval"]["rp_seed_200"] = evaluate(rp_case(200), nf, rp_case(200)(nf)["simulation"]["t_end"], params)
    _log("evaluated rp_seed_200", t0)
    report["eval"]["bubble_heldout"] = evaluate(sb_case((0.42, 0.55), 0.2, 0.2), nf, 0.2, params)
    _log("evaluated bubble_heldout", t0)
    with open(args.out, "w") as fh:
        json.dump(report, fh, indent=1)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
