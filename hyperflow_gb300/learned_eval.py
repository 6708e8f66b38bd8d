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
from .learned import (LearnedSolver, change_weights, evaluate_learned, evaluate_plain, fine_sequence,
                      init_params, one_step_loss, train, train_rollout)


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
    ap.add_argument("--stride", type=int, default=8, help="pairs mode: every stride-th window")
    ap.add_argument("--modes", default="pairs,roll4",
                    help="comma list of training modes: pairs (one-step pairs from the filtered "
                         "fine runs), gpairs (the same, trained with the guard applied) or rollK (one-step training on the solver's own states after "
                         "up to K of its steps)")
    ap.add_argument("--bounds", default="0.5,local",
                    help="comma list of guards to evaluate each model with: a number is the change "
                         "bound, 'local' the local-extremum bounds")
    ap.add_argument("--extra-cases", type=int, default=0,
                    help="additional training cases: this many more Riemann seeds (102, 103, ...) and "
                         "as many more bubble placements")
    ap.add_argument("--out", default="learned_report.json")
    args = ap.parse_args()
    nf, f = args.n_fine, 4
    nc = nf // f
    report = {"n_fine": nf, "n_coarse": nc, "iters": args.iters, "lr": args.lr}
    t0 = time.perf_counter()
    train_sets = [("rp_seed_100", rp_case(100), None), ("rp_seed_101", rp_case(101), None),
                  ("bubble_a", sb_case((0.4, 0.5), 0.2, 1.0), 0.25),
                  ("bubble_b", sb_case((0.45, 0.45), 0.2, 1.0), 0.25)]
    rng = np.random.default_rng(1)
    for k in range(args.extra_cases):
        train_sets.append((f"rp_seed_{102 + k}", rp_case(102 + k), None))
        bx, by = float(rng.uniform(0.35, 0.5)), float(rng.uniform(0.4, 0.6))
        r = float(rng.uniform(0.15, 0.22))
        train_sets.append((f"bubble_{k}", sb_case((bx, by), r, 1.0), 0.25))
    seqs = []
    for name, fn, t_end in train_sets:
        c = fn(nf)
        T = t_end if t_end is not None else c["simulation"]["t_end"]
        seqs.append(fine_sequence(c, T, factor=f))
        _log(f"fine data {name}: {len(seqs[-1][1])} windows", t0)
    pairs = [(st[k], st[k + 1], dts[k]) for st, dts in seqs for k in range(len(dts))]
    report["train_windows"] = len(pairs)
    report["data_seconds"] = time.perf_counter() - t0
    held = [fine_sequence(rp_case(200)(nf), rp_case(200)(nf)["simulation"]["t_end"], factor=f),
            fine_sequence(cases.shock_bubble_case(nf, bubble=(0.42, 0.55)), 0.2, factor=f)]
    held_pairs = [(st[k], st[k + 1], dts[k]) for st, dts in held for k in range(0, len(dts), 4)]
    _log(f"held-out data: {len(held_pairs)} pairs", t0)
    evals = {"rp_seed_200": (rp_case(200), rp_case(200)(nf)["simulation"]["t_end"]),
             "bubble_heldout": (sb_case((0.42, 0.55), 0.2, 0.2), 0.2)}
    report["eval"] = {}
    base = {}
    for name, (fn, t_end) in evals.items():
        res, ref, U0 = evaluate_plain(fn, nf, t_end, factor=f)
        report["eval"][name] = res
        base[name] = (ref, U0, t_end)
    _log("plain runs evaluated", t0)
    w = change_weights(pairs)
    report["models"] = {}
    for mode in args.modes.split(","):
        # mode[:iterations[:learning rate]]
        parts = mode.split(":")
        kind = parts[0]
        iters = int(parts[1]) if len(parts) > 1 else args.iters
        lr = float(parts[2]) if len(parts) > 2 else args.lr
        ls = LearnedSolver(nc, 1.0 / nc)
        ls.set_params(init_params(0))
        if kind == "gpairs":          # pairs, trained with the change guard (bound 2) applied
            ls.set_bound(2.0)
            ls.set_train_guard(True)
            kind = "pairs"
        t1 = time.perf_counter()
        if kind == "pairs":
            sub = pairs[::args.stride]
            losses, _ = train(ls, sub, iters, lr=lr, w=w)
        elif kind.startswith("roll"):
            losses, _ = train_rollout(ls, seqs, iters, lr=lr, max_roll=int(kind[4:]), w=w)
        else:
            raise SystemExit(f"unknown mode {mode}")
        m = {"train_seconds": time.perf_counter() - t1,
             "train_loss_first100": float(losses[:100].mean()),
             "train_loss_last100": float(losses[-100:].mean()),
             "heldout_one_step_loss": {"plain": one_step_loss(ls, held_pairs, w, False),
                                       "learned": one_step_loss(ls, held_pairs, w, True)}}
        params = ls.params()
        ls.close()
        np.save(args.out.replace(".json", f"_{mode.replace(':', '_')}_params.npy"), params)
        m["eval"] = {}
        for guard in args.bounds.split(","):
            kw = {"guard_mode": 1} if guard == "local" else {"bound": float(guard)}
            tag = "guard_local" if guard == "local" else f"bound_{float(guard):g}"
            try:
                ev = {name: evaluate_learned(t_end, params, ref, U0, **kw)
                      for name, (ref, U0, t_end) in base.items()}
            except Exception as e:   # a run the guard let blow up
                ev = {"failed": str(e)}
            m["eval"][tag] = ev
            _log(f"model {mode}, {tag}: " +
                 ", ".join(f"{k} l1 {v['l1_rho']:.5f}" if isinstance(v, dict) else f"{k} {v}"
                           for k, v in ev.items()), t0)
        report["models"][mode] = m
    with open(args.out, "w") as fh:
        json.dump(report, fh, indent=1)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
