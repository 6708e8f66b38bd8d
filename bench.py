#!/usr/bin/env python
"""Benchmark of the plain FP64 MUSCL-Hancock + HLLC time step on one GB300.

Workload: the Mach 3 forward-facing step, 3 blocks at dx = dy = 1/1365 (819x273,
819x1092, 3276x1092 = 4,695,327 cells), MinBee limiter, CFL 0.8, uniform inflow start.
One step = ghost fill + CFL dt + the three block updates (each with its own predictor
TimeStep call), exactly the reference's step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput (state in HBM,
CUDA events on the solver's stream around K steps); `e2e` is the same metric through the
C ABI with host buffers (per step, hf_step_io on pinned host memory: the kernels read every
block from the host buffers, step, and the stencils store the updated cells straight back to
them, so the download overlaps the updates).  With --gpus N under torchrun, every rank runs an
independent replica (the path does not shard across GPUs) and `value` sums the replicas.

Other workloads (`--workload`, one JSON line each, not the headline):
    square    one N x N four-quadrant block (--n, --scheme, --limiter)
    batch     512 batched Riemann problems in one persistent launch (autotuned)
    uns       the ~1M-triangle channel, edge-based (or --uns-per-side) fluxes
    quad256   the 256^2 Godunov problem as a batch of one (the whole run one launch)
    learned   the 512^2 learned coarse step (FP32 + the tcgen05 MLP on every face)
    learned-train  a 512^2 training iteration of the learned solver (tcgen05 forward and backward)
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_CELL = 64          # 4 FP64 read + 4 FP64 written per cell update
WORKLOAD = "mach3_forward_facing_step_3block_dx1_1365_muscl_hancock_minbee_hllc_fp64"


def make_case(limiter: str = "MinBee", workload: str = "ffs", n: int = 4096, scheme: str = "MUSCLHancock"):
    from hyperflow_gb300 import cases
    if workload == "square":
        if scheme == "Godunov":
            return cases.quadrant_case(n, scheme="Godunov", cfl=0.8)
        return cases.quadrant_case(n, scheme="MUSCLHancock", limiter=limiter, cfl=0.8)
    return cases.forward_facing_step_case(1365, limiter=limiter, cfl=0.8, t_end=4.0)


def workload_name(args):
    if args.workload == "square":
        if args.scheme == "Godunov":
            return f"quadrant_riemann_{args.n}x{args.n}_godunov_hllc_fp64"
        return f"quadrant_riemann_{args.n}x{args.n}_muscl_hancock_{args.limiter.lower()}_hllc_fp64"
    return WORKLOAD if args.limiter == "MinBee" else WORKLOAD.replace("minbee", args.limiter.lower())


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per cell update of the stencil kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "mh_step_kernel_ffs_traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return None


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_value(ms: float, ws: int, cells: int, steps: int, pg=None, device="cuda"):
    """Whole-job throughput of N independent replicas: the slowest rank's time bounds the job
    (max over ranks), and every rank updated `cells` cells per step.  Returns (Mcell-updates/s,
    the max time in ms)."""
    t_max = ms
    if pg is not None:
        import torch
        tt = torch.tensor([ms], dtype=torch.float64, device=device)
        pg.all_reduce(tt, op=pg.ReduceOp.MAX)
        t_max = float(tt.item())
    return ws * cells * steps / (t_max / 1e3) / 1e6, t_max


def cpu_run(case, steps: int, nthreads: int):
    """The oracle (C restatement of the reference step) on host cores."""
    from oracle.oracle import Oracle, build_port
    build_port()
    o = Oracle(case, nthreads=nthreads)
    t0 = time.perf_counter()
    o.run(steps)
    return time.perf_counter() - t0


def reference_cpu_baseline(limiter: str, seconds: float = 10.0):
    """The reference's own solver -- its sources compiled serially (oracle/_ref, from the reference
    tree or its staged copy) -- on one host core, timed on the forward-facing step at a reduced
    spacing (dx = 1/200: 100,800 cells; at the benchmark's spacing its per-cell allocations need
    about 4 GB and minutes per step): a bounded sample of whole steps, after one untimed step."""
    from hyperflow_gb300 import cases
    from oracle import oracle
    if not oracle.ref_available():
        return None
    case = cases.forward_facing_step_case(200, limiter=limiter, cfl=0.8, t_end=4.0)
    cells = sum(b["x_cells"] * b["y_cells"] for b in case["mesh"]["blocks"])
    ref = oracle.RefCart(case)
    ref.run(1)
    t0 = time.perf_counter()
    ref.run(1)
    probe = time.perf_counter() - t0
    n = int(max(1, min(100, seconds / max(probe, 1e-3))))
    t0 = time.perf_counter()
    ref.run(n)
    el = time.perf_counter() - t0
    return {"value": cells * n / el / 1e6, "unit": "Mcell-updates/s", "cores": 1, "kind": "reference",
            "sample": f"{n} steps of the forward-facing step at dx = 1/200 ({cells} cells), "
                      f"{limiter}, after 2 steps; the reference's sources compiled serially (-O3)"}


def reference_arm(args, cells):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    case = make_case(args.limiter, args.workload, args.n, args.scheme)
    nth = os.cpu_count() or 1
    from oracle.oracle import Oracle, build_port
    build_port()
    o = Oracle(case, nthreads=nth)
    o.run(args.warmup)
    t0 = time.perf_counter()
    o.run(args.steps)
    el = time.perf_counter() - t0
    v = cells * args.steps / el / 1e6
    print(json.dumps({
        "metric": "Mcell-updates/s", "value": v, "unit": "Mcell-updates/s", "impl": "reference",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the case's own initial condition)",
        "config": {"workload": workload_name(args), "cells": cells},
        "cpu_baseline": {"value": v, "unit": "Mcell-updates/s", "cores": nth, "kind": "port",
                         "sample": f"{args.steps} full steps of the workload after {args.warmup} warm-up steps"},
        "e2e": {"value": v, "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def timed_device(stream, fn):
    """CUDA-event milliseconds of fn() on `stream` (synchronised on both sides)."""
    import torch
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def bench_batch(args):
    """The batched workload: 512 seeded four-quadrant Riemann problems (sides log-uniform in
    64..1024), MUSCL-Hancock MinBee, per-instance dt, autotuned launch shape, the run of
    `steps` steps in one persistent launch captured in a CUDA graph."""
    import numpy as np  # noqa: F401
    import torch
    from hyperflow_gb300 import BatchSolver, cases
    from oracle.oracle import Oracle, build_port
    m = cases.batch_manifest(args.instances, seed=0)
    b = BatchSolver(m)
    if args.batch_config >= 0:
        b.set_config(args.batch_config)
        best, trial_ms = args.batch_config, []
    else:
        best, trial_ms = b.autotune(steps_per_trial=2)
    stream = torch.cuda.ExternalStream(b.stream())
    b.run(args.warmup, graph=True)
    b.sync()
    with Clocks(0) as clk:
        ms = timed_device(stream, lambda: b.run(args.steps, graph=True))
    b.sync()
    cells = b.total_cells
    value = cells * args.steps / (ms / 1e3) / 1e6
    hbm, peak_kind = peaks()
    achieved = BYTES_PER_CELL * cells * args.steps / (ms / 1e3) / 1e9
    # CPU baseline: the oracle on all host cores over a bounded sample of the instances
    build_port()
    nth = os.cpu_count() or 1
    sample = list(range(0, args.instances, 16))
    sample_cells, t0 = 0, time.perf_counter()
    for i in sample:
        o = Oracle(m["cases"][i], nthreads=nth)
        o.run(20)
        sample_cells += 20 * m["cases"][i]["mesh"]["blocks"][0]["x_cells"] ** 2
    cpu_s = time.perf_counter() - t0
    print(json.dumps({
        "metric": "Mcell-updates/s", "value": value, "unit": "Mcell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded four-quadrant Riemann problems)",
        "config": {"workload": f"batched_{args.instances}_quadrant_riemann_sides_64_1024_muscl_hancock_minbee_hllc_fp64",
                   "instances": args.instances, "cells": cells, "cfl": cases.CFL_2D, "autotuned_config": best,
                   "autotune_trial_ms": [float(x) for x in trial_ms],
                   "l2": "state 2 x %.0f MB > 129 MB L2, no flush needed" % (cells * 32 / 1e6)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": None, "peak_kind": peak_kind,
                     "kernel": "batch_kernel<MUSCL-Hancock> (persistent, all instances, one launch per run)"},
        "cpu_baseline": {"value": sample_cells / cpu_s / 1e6, "unit": "Mcell-updates/s", "cores": nth,
                         "kind": "port", "sample": f"every 16th instance ({len(sample)}), 20 steps each"},
        "e2e": None, "gpu_launches": 1, "clocks": clk.summary()}), flush=True)
    b.close()


def bench_quad256(args):
    """The reference's first configuration: the 256^2 four-quadrant Riemann problem, Godunov +
    HLLC, CFL 0.8, `steps` steps (200 in the reference's run).  At 65,536 cells a step is too
    small to fill the GPU through per-step launches, so the whole run goes through the batched
    path as a batch of one: one persistent launch, grid barriers between steps.  The per-block
    solver's device loop (CUDA graph of the per-step launches) is timed beside it."""
    import torch
    from hyperflow_gb300 import BatchSolver, CartSolver, cases
    from oracle.oracle import Oracle, build_port
    case = cases.quadrant_case(256)
    b = BatchSolver({"cases": [case]})
    best, trial_ms = b.autotune(steps_per_trial=20)
    stream = torch.cuda.ExternalStream(b.stream())
    b.run(args.warmup, graph=True)
    b.sync()
    with Clocks(0) as clk:
        ms = timed_device(stream, lambda: b.run(args.steps, graph=True))
    b.sync()
    cells = 256 * 256
    value = cells * args.steps / (ms / 1e3) / 1e6
    s = CartSolver(case)
    s.run(args.warmup)
    sstream = torch.cuda.ExternalStream(s.stream())
    ms_pb = timed_device(sstream, lambda: s.run(args.steps, graph=True))
    hbm, peak_kind = peaks()
    achieved = BYTES_PER_CELL * cells * args.steps / (ms / 1e3) / 1e9
    build_port()
    nth = os.cpu_count() or 1
    o = Oracle(case, nthreads=nth)
    t0 = time.perf_counter()
    o.run(args.steps)
    cpu_s = time.perf_counter() - t0
    print(json.dumps({
        "metric": "Mcell-updates/s", "value": value, "unit": "Mcell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the case's own initial condition)",
        "config": {"workload": "quadrant_riemann_256x256_godunov_hllc_fp64", "cells": cells, "cfl": 0.8,
                   "path": "batch of one: one persistent launch for the whole run", "autotuned_config": best,
                   "l2": "state 2 x 2 MB, L2-resident by nature across the steps of the one launch"},
        "per_block_device_loop_value": cells * args.steps / (ms_pb / 1e3) / 1e6,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": None, "peak_kind": peak_kind,
                     "kernel": "batch_kernel<Godunov> (persistent)"},
        "cpu_baseline": {"value": cells * args.steps / cpu_s / 1e6, "unit": "Mcell-updates/s", "cores": nth,
                         "kind": "port", "sample": f"the whole run ({args.steps} steps)"},
        "e2e": None, "gpu_launches": 1, "clocks": clk.summary()}), flush=True)
    b.close()
    s.close()


def bench_learned(args):
    """The learned coarse solver's step: 512^2 FP32 MUSCL-Hancock MinBee + HLLC with the MLP
    face-flux correction (features -> 64 -> 64 -> 4, BF16 on the tensor cores, FP32
    accumulation) on every face, random-init weights (throughput does not depend on them), the
    change guard on.  Steps are enqueued without reading back the rejection count and timed
    with CUDA events on the solver's stream: with the fused face kernel (the line's value), with
    the plain flux fused in as well, with the separate kernels, and without the MLP; the MLP
    path's throughput is its FLOPs over the time it adds to a step."""
    import numpy as np
    import torch
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import LearnedSolver, init_params
    n = 512
    case = cases.quadrant_case(n, scheme="MUSCLHancock", limiter="MinBee", cfl=cases.CFL_2D)
    s = CartSolver(case)
    U0 = s.state(0)[:, 2:-2, 2:-2].astype(np.float32)
    s.close()
    ls = LearnedSolver(n, 1.0 / n, cfl=cases.CFL_2D)
    ls.set_params(init_params(0))
    ls.set_bound(0.5)
    stream = torch.cuda.ExternalStream(ls.stream())

    def timed(use_mlp, fused=1):
        ls.set_fused(fused)
        ls.set_state(U0)
        dt = ls.cfl_dt()
        for _ in range(args.warmup):
            ls.step(dt, use_mlp, count_rejected=False)
        return timed_device(stream, lambda: [ls.step(dt, use_mlp, count_rejected=False) for _ in range(args.steps)])

    with Clocks(0) as clk:
        ms_mlp = timed(True)
    ms_plain = timed(False)
    ms_unfused = timed(True, fused=0)
    ms_flux_fused = timed(True, fused=2)
    cells = n * n
    faces = 2 * n * (n + 1)
    flop = 16896.0 * faces * args.steps            # 2 x (64x64 + 64x64 + 64x4) per face, x 2 (FMA)
    extra_s = max(ms_mlp - ms_plain, 1e-9) / 1e3
    achieved = flop / extra_s / 1e12
    peak = 1947.2
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            peak = float(json.load(f).get("bf16_tflops", peak))
    print(json.dumps({
        "metric": "Mcell-updates/s", "value": cells * args.steps / (ms_mlp / 1e3) / 1e6, "unit": "Mcell-updates/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mlp / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32 + bf16 MLP",
        "data": "synthetic (the 512^2 quadrant Riemann problem; random-init MLP weights)",
        "config": {"workload": "learned_coarse_512x512_muscl_hancock_minbee_mlp_flux_correction", "cells": cells,
                   "faces": faces, "mlp": "features->64->64->4 GELU, BF16 weights, FP32 accumulation"},
        "plain_fp32_value": cells * args.steps / (ms_plain / 1e3) / 1e6,
        "unfused_value": cells * args.steps / (ms_unfused / 1e3) / 1e6,
        "flux_fused_value": cells * args.steps / (ms_flux_fused / 1e3) / 1e6,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None, "peak_kind": "measured",
                     "kernel": "face_kernel (per 128-face tile: features, the tcgen05.mma kind::f16 MLP with "
                               "TMEM accumulators, the corrections); achieved = MLP FLOPs over the time the MLP "
                               "path adds to a step"},
        "cpu_baseline": None, "e2e": None, "gpu_launches": None, "clocks": clk.summary()}), flush=True)
    ls.close()


def bench_uns(args):
    """The unstructured workload: ~1M triangles of a jittered-lattice Delaunay mesh of
    [0,4]x[0,2] minus a disc, Mach 2 inflow, CFL 0.5, Godunov + HLLC, edge-based fluxes,
    `steps` steps in the device loop (CUDA graph)."""
    import tempfile
    import numpy as np
    import torch
    from hyperflow_gb300 import UnsSolver, meshgen
    from oracle import oracle
    V, codes = meshgen.jittered_hole_mesh(1_000_000, seed=0)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "channel.hmsh")
        meshgen.write_hmsh(path, V, codes)
        case = meshgen.channel_case(path, cfl=0.5)
        s = UnsSolver(case)
    s.set_edge_mode(not args.uns_per_side)
    stream = torch.cuda.ExternalStream(s.stream())
    s.run(args.warmup)
    with Clocks(0) as clk:
        ms = timed_device(stream, lambda: s.run(args.steps))
    cells = s.ncells
    m = s.mesh_arrays()
    nedges = int((m["nbr"] >= 0).sum() // 2 + (m["nbr"] < 0).sum())
    value = cells * args.steps / (ms / 1e3) / 1e6
    hbm, peak_kind = peaks()
    achieved = (64 * cells + 40 * nedges) * args.steps / (ms / 1e3) / 1e9
    nth = os.cpu_count() or 1
    U = np.zeros((4, cells))
    U[:] = oracle.prim_to_cons(case["initial_condition"]["init_state"])[:, None]
    inlet = oracle.prim_to_cons(case["mesh"]["boundaries"]["inlet"])
    n_cpu = 20
    t0 = time.perf_counter()
    oracle.uns_run(1.4, 0.5, 0, m["pair_start"], m["nbr"], m["angle"], m["length"], m["area"], m["rin"],
                   inlet, U, n_cpu, nthreads=nth)
    cpu_s = time.perf_counter() - t0
    print(json.dumps({
        "metric": "Mcell-updates/s", "value": value, "unit": "Mcell-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded jittered-lattice Delaunay mesh, uniform Mach 2 start)",
        "config": {"workload": "unstructured_1M_triangles_hole_channel_godunov_hllc_fp64",
                   "cells": cells, "unique_edges": nedges, "cfl": 0.5,
                   "flux": "per (cell, edge) pair" if args.uns_per_side else "edge-based"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": None, "peak_kind": peak_kind,
                     "kernel": "uns_step_kernel (+ uns_edge_flux_kernel)"},
        "cpu_baseline": {"value": cells * n_cpu / cpu_s / 1e6, "unit": "Mcell-updates/s", "cores": nth,
                         "kind": "port", "sample": f"first {n_cpu} steps, per-pair fluxes"},
        "e2e": None, "gpu_launches": 4 * args.steps, "clocks": clk.summary()}), flush=True)
    s.close()


def bench_learned_train(args):
    """Training iterations of the learned coarse solver at 512^2: forward with the activations
    saved (tcgen05), loss and its gradient, the backward (tcgen05 weight gradients), Adam --
    each on a state of the 512^2 quadrant Riemann problem against a slightly perturbed target,
    the iteration's loss read back (a wait per iteration, as training does)."""
    import numpy as np
    import torch
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import LearnedSolver, init_params
    n = 512
    s = CartSolver(cases.quadrant_case(n, scheme="MUSCLHancock", limiter="MinBee", cfl=cases.CFL_2D))
    U0 = s.state(0)[:, 2:-2, 2:-2].astype(np.float32)
    s.close()
    ls = LearnedSolver(n, 1.0 / n, cfl=cases.CFL_2D)
    ls.set_params(init_params(0))
    w = np.ones(4, np.float32)
    T = U0 * np.float32(1.001)
    ls.set_state(U0)
    dt = ls.cfl_dt()
    for _ in range(args.warmup):
        ls.train_step(U0, T, w, dt, 1e-4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ls.train_step(None, T, w, dt, 1e-4)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    print(json.dumps({
        "metric": "ms per training iteration", "value": ms, "unit": "ms", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": False, "dtype": "fp32 + bf16 MLP",
        "data": "synthetic (the 512^2 quadrant Riemann problem, target scaled by 1.001)",
        "config": {"workload": "learned_training_iteration_512x512", "faces": 2 * n * (n + 1)}}), flush=True)


def state_note(args, t_start: float) -> str:
    if args.pre_steps > 0:
        return f"developed flow: timed from t = {t_start:.4g}, after {args.pre_steps} untimed steps"
    return "from the initial condition (first steps of the run)"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--limiter", default="MinBee", choices=["MinBee", "VanLeer"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU-baseline sample budget")
    ap.add_argument("--workload", default="ffs",
                    choices=["ffs", "square", "batch", "uns", "quad256", "learned", "learned-train"],
                    help="ffs: the 3-block forward-facing step (default); square: one n x n block; "
                         "batch: 512 batched Riemann problems; uns: the 1M-triangle channel")
    ap.add_argument("--instances", type=int, default=512, help="batch workload: number of instances")
    ap.add_argument("--batch-config", type=int, default=-1,
                    help="batch workload: this launch configuration instead of the autotuner's choice")
    ap.add_argument("--uns-per-side", action="store_true",
                    help="uns workload: per-(cell, edge) fluxes (bit-exact mode) instead of edge-based")
    ap.add_argument("--n", type=int, default=4096, help="side of the square workload")
    ap.add_argument("--scheme", default="MUSCLHancock", choices=["MUSCLHancock", "Godunov"],
                    help="scheme of the square workload")
    ap.add_argument("--per-block-launches", action="store_true",
                    help="ffs/square workloads: one stencil launch per block instead of the all-blocks launch")
    ap.add_argument("--pre-steps", type=int, default=0,
                    help="ffs/square workloads: untimed steps before the warm-up, so that the timed steps see a "
                         "developed flow instead of the initial condition")
    ap.add_argument("--developed-steps", type=int, default=10000,
                    help="ffs workload, full run: after the main measurement, advance this many untimed steps "
                         "and time --steps more on the developed flow (0: skip)")
    ap.add_argument("--quick", action="store_true",
                    help="device-resident timing only (no graph pass, e2e or CPU baseline)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.workload in ("batch", "uns", "quad256", "learned", "learned-train"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference arm is timed on the forward-facing step and square workloads"}))
            return
        import numpy as np  # noqa: F401
        import torch
        torch.cuda.set_device(0)
        {"batch": bench_batch, "uns": bench_uns, "quad256": bench_quad256, "learned": bench_learned,
         "learned-train": bench_learned_train}[args.workload](args)
        return

    from hyperflow_gb300 import cases
    case = make_case(args.limiter, args.workload, args.n, args.scheme)
    cells = cases.total_cells(case)

    if args.impl == "reference":
        reference_arm(args, cells)
        return

    import numpy as np
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    from hyperflow_gb300 import CartSolver
    s = CartSolver(case)
    nb = s.nblocks
    s.set_block_launches(args.per_block_launches)
    stream = torch.cuda.ExternalStream(s.stream())

    # ---- device-resident timed region ----
    if args.pre_steps > 0:
        s.run(args.pre_steps, graph=True)
        s.sync()
    t_start = s.time()[0]
    s.run(args.warmup, graph=False)
    s.sync()
    s.profile(True)          # events around every step's stencil launches (same stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    with Clocks(local) as clk:
        e0.record(stream)
        s.run(args.steps, graph=False)
        e1.record(stream)
        torch.cuda.synchronize()
    s.sync()
    ms = e0.elapsed_time(e1)
    stencil_ms, stencil_launches = s.kernel_time(0)
    s.profile(False)
    value, t_max = replica_value(ms, ws, cells, args.steps, pg)
    hllc_fallbacks = s.hllc_errors()
    reruns = s.blocks_rerun()

    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": "Mcell-updates/s", "value": value, "unit": "Mcell-updates/s",
                              "steps": args.steps, "ms_per_step": t_max / args.steps,
                              "config": {"workload": workload_name(args), "cells": cells,
                                         "state": state_note(args, t_start)},
                              "stencil_ms_per_step": stencil_ms / args.steps,
                              "blocks_rerun": reruns}), flush=True)
        s.close()
        return

    # same run through the CUDA graph (one captured step replayed K times)
    s.run(1, graph=True)
    barrier()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    s.run(args.steps, graph=True)
    g1.record(stream)
    torch.cuda.synchronize()
    graph_value = cells * args.steps / (g0.elapsed_time(g1) / 1e3) / 1e6

    # ---- end to end through the C ABI with host buffers ----
    host = []
    h2d = 0
    for b in range(nb):
        d = s.block_dims(b)
        t = torch.empty((4, d["total_y"], d["total_x"]), dtype=torch.float64).pin_memory()
        a = t.numpy()
        s.state(b, out=a)
        host.append((t, a))
        h2d += a.nbytes
    e2e_steps = max(3, min(args.steps, 30))
    arrays = [h[1] for h in host]
    direct = all(s.host_mapped(a) for a in arrays)
    s.step_io(arrays)              # warm-up: loads the host-buffer kernels
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.step_io(arrays)          # upload all blocks, one step, download all blocks
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = ws * cells * e2e_steps / e2e_s / 1e6

    # ---- the same steps on a developed flow: the bow shock, reflections and subsonic regions put
    # HLLC star states on many more faces than the uniform inflow the run starts from ----
    developed = None
    if args.workload == "ffs" and args.developed_steps > 0:
        s.run(args.developed_steps, graph=True)
        s.sync()
        t_dev = s.time()[0]
        s.run(args.warmup, graph=False)
        barrier()
        d0 = torch.cuda.Event(enable_timing=True)
        d1 = torch.cuda.Event(enable_timing=True)
        d0.record(stream)
        s.run(args.steps, graph=False)
        d1.record(stream)
        torch.cuda.synchronize()
        s.sync()
        dms = d0.elapsed_time(d1)
        developed = {"value": cells * args.steps / (dms / 1e3) / 1e6, "unit": "Mcell-updates/s",
                     "ms_per_step": dms / args.steps, "t_start": t_dev, "untimed_steps": args.developed_steps}

    # ---- roofline of the stencil kernel ----
    hbm, peak_kind = peaks()
    achieved = BYTES_PER_CELL * cells * args.steps / (stencil_ms / 1e3) / 1e9
    traffic = None
    tr = ncu_traffic()
    tiles = sum(-(-b["x_cells"] // 32) * -(-b["y_cells"] // 12) for b in case["mesh"]["blocks"])
    all_blocks = (args.scheme == "MUSCLHancock" and nb <= 4 and not args.per_block_launches
                  and (nb > 1 or tiles >= 1024))
    per_launch = 1 if all_blocks else nb           # stencil launches per step
    if tr and tr.get("workload") == workload_name(args):
        traffic = tr["dram_bytes_per_cell_update"] * cells / per_launch
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": BYTES_PER_CELL * cells / per_launch,
            "avg_launch_ms": stencil_ms / max(stencil_launches * per_launch, 1),
            "kernel": ("mh_step_kernel (every block of the step in one launch: fused MUSCL-Hancock + HLLC + "
                       "forward Euler + CFL epilogue)") if all_blocks else
                      "mh_kernel (fused MUSCL-Hancock + HLLC + forward Euler + CFL epilogue)"}
    # the bound that binds on this part: FP64 issue (2 lanes per SM per clock)
    if tr and tr.get("workload") == workload_name(args) and tr.get("fp64_ops_per_cell_update"):
        sm_mhz = 2070.0
        pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pk):
            with open(pk) as f:
                sm_mhz = float(json.load(f).get("sm_max_mhz", sm_mhz))
        nsm = torch.cuda.get_device_properties(local).multi_processor_count
        ops = tr["fp64_ops_per_cell_update"] * cells * args.steps / (stencil_ms / 1e3) / 1e9
        peak_ops = 2.0 * nsm * sm_mhz / 1e3
        roof["fp64_pipe"] = {"achieved": ops, "peak": peak_ops, "unit": "G FP64 ops/s (FMA = 1)",
                             "frac": ops / peak_ops,
                             "ops_per_cell_update": tr["fp64_ops_per_cell_update"]}

    # ---- CPU baseline (rank 0, N=1): the oracle on all host cores, bounded sample ----
    cpu = None
    if rank == 0 and ws == 1:
        nth = os.cpu_count() or 1
        probe = cpu_run(case, 1, nth)
        n_cpu = int(max(1, min(200, args.cpu_seconds / max(probe, 1e-3))))
        el = cpu_run(case, n_cpu, nth)
        cpu = {"value": cells * n_cpu / el / 1e6, "unit": "Mcell-updates/s", "cores": nth,
               "kind": "port",
               "sample": f"first {n_cpu} steps of the same workload (all {cells} cells)"}

    cpu_ref = None
    if rank == 0 and ws == 1 and args.workload == "ffs" and args.cpu_seconds > 0:
        cpu_ref = reference_cpu_baseline(args.limiter)

    # step start, the ghost fill + ghost CFL + dt, the stencils (one launch for every block of a
    # MUSCL-Hancock mesh of up to 4 blocks, else one per block), finalize
    launches_per_step = 3 + per_launch
    if rank == 0:
        line = {
            "metric": "Mcell-updates/s", "value": value, "unit": "Mcell-updates/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (the case's own initial condition: uniform Mach 3 inflow)",
            "config": {"workload": workload_name(args), "cells": cells, "blocks": nb, "limiter": args.limiter,
                       "state": state_note(args, t_start),
                       "cfl": 0.8, "l2": "state 2 x 151 MB buffers > 129 MB L2, no flush needed",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "roofline": roof,
            "cpu_baseline": cpu,
            "cpu_baseline_reference": cpu_ref,
            "e2e": {"value": e2e_value, "unit": "Mcell-updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": h2d, "steps": e2e_steps,
                    "path": "kernels read and write pinned host buffers" if direct else "copies"},
            "gpu_launches": launches_per_step * args.steps,
            "stencil_ms_per_step": stencil_ms / args.steps,
            "non_stencil_ms_per_step": t_max / args.steps - stencil_ms / args.steps,
            "developed": developed,
            "clocks": clk.summary(),
            "graph_value": graph_value,
            "hllc_zero_flux_fallbacks": hllc_fallbacks,
            "blocks_rerun": reruns,
        }
        print(json.dumps(line), flush=True)
    s.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
