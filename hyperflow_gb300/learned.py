"""Learned coarse solver: host driver for the kernels of include/hyperflow_gb300_learned.h.

* ``LearnedSolver``: one coarse n x n FP32 grid (MUSCL-Hancock + HLLC) with the MLP flux
  correction, its parameters, and training on the device.
* ``fine_pairs``: training pairs generated by the plain FP64 solver itself (``CartSolver``)
  on the fine grid, box-filtered by ``factor``: (coarse state, filtered state after
  ``factor`` fine steps, the summed fine dt).
* ``evaluate``: L1 density error against the filtered FP64 fine solution, and wall time, of
  the plain and learned coarse runs next to plain FP64 runs at 2x and 4x resolution.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from ._lib import check, lib
from .solver import CartSolver

_MSG = "hf_lc_last_error_message"
NPARAM = 64 * 64 + 64 + 64 * 64 + 64 + 4 * 64 + 4


def init_params(seed: int = 0, out_scale: float = 1e-3) -> np.ndarray:
    """Scaled-uniform hidden layers; a small output layer so training starts from the
    plain scheme (corrections near zero)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, np.float32)
    o = 0
    for fan_in, fan_out, scale in ((64, 64, 1.0), (64, 64, 1.0), (64, 4, out_scale)):
        lim = scale * np.sqrt(6.0 / (fan_in + fan_out))
        p[o:o + fan_in * fan_out] = rng.uniform(-lim, lim, fan_in * fan_out)
        o += fan_in * fan_out + fan_out
    return p


def box_filter(U: np.ndarray, k: int) -> np.ndarray:
    """Cell averages over k x k blocks of a [4][n][n] state (conservative)."""
    v, ny, nx = U.shape
    return U.reshape(v, ny // k, k, nx // k, k).mean(axis=(2, 4))


class LearnedSolver:
    def __init__(self, n: int, dx: float, gamma: float = 1.4, cfl: float = 0.4, limiter: int = 0):
        L = lib()
        h = C.c_void_p()
        st = L.hf_lc_create(n, dx, gamma, cfl, limiter, C.byref(h))
        self._h = h
        if st != 0:
            try:
                check(st, h, _MSG)
            finally:
                if h:
                    L.hf_lc_destroy(h)
                self._h = None
        self.n = n

    def close(self):
        if getattr(self, "_h", None):
            lib().hf_lc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, st):
        check(st, self._h, _MSG)

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == NPARAM
        self._c(lib().hf_lc_set_params(self._h, p.ctypes.data))

    def params(self) -> np.ndarray:
        p = np.empty(NPARAM, np.float32)
        self._c(lib().hf_lc_get_params(self._h, p.ctypes.data))
        return p

    def set_bound(self, b: float):
        self._c(lib().hf_lc_set_bound(self._h, b))

    def set_train_guard(self, on: bool):
        """training steps apply the guard as inference does"""
        self._c(lib().hf_lc_set_train_guard(self._h, int(on)))

    def set_fused(self, mode: int, ctas_per_sm: int = 0):
        """how inference steps run: 1 (default) features + MLP + corrections in one kernel, 2 the
        plain fluxes in it too, 0 separate kernels -- the same results bit for bit; ctas_per_sm
        sets the fused kernel's launch shape (0: as many as fit)"""
        self._c(lib().hf_lc_set_fused(self._h, int(mode), int(ctas_per_sm)))

    def set_guard_mode(self, mode: int):
        """0: change bound (set_bound); 1: local-extremum (flux-corrected transport) bounds"""
        self._c(lib().hf_lc_set_guard_mode(self._h, mode))

    def set_state(self, U, t: float = 0.0):
        U = np.ascontiguousarray(U, dtype=np.float32)
        assert U.shape == (4, self.n, self.n)
        self._c(lib().hf_lc_set_state(self._h, U.ctypes.data))
        self._c(lib().hf_lc_set_time(self._h, t))

    def state(self) -> np.ndarray:
        U = np.empty((4, self.n, self.n), np.float32)
        self._c(lib().hf_lc_get_state(self._h, U.ctypes.data))
        return U

    def cfl_dt(self) -> float:
        d = C.c_double()
        self._c(lib().hf_lc_cfl_dt(self._h, C.byref(d)))
        return d.value

    def step(self, dt: float, use_mlp: bool, count_rejected: bool = True):
        """one step; returns the cells whose corrections the guard rejected (a wait for the
        step), or None with count_rejected False (the step is only enqueued)"""
        if not count_rejected:
            self._c(lib().hf_lc_step(self._h, dt, int(use_mlp), None))
            return None
        r = C.c_int64()
        self._c(lib().hf_lc_step(self._h, dt, int(use_mlp), C.byref(r)))
        return r.value

    def run_to(self, t_end: float, use_mlp: bool):
        k, r = C.c_int64(), C.c_int64()
        self._c(lib().hf_lc_run_to(self._h, t_end, int(use_mlp), C.byref(k), C.byref(r)))
        return k.value, r.value

    def train_step(self, U0, T, w, dt: float, lr: float) -> float:
        """U0 None: from the current device state (kept)."""
        ptr = None
        if U0 is not None:
            U0 = np.ascontiguousarray(U0, dtype=np.float32)
            ptr = U0.ctypes.data
        T = np.ascontiguousarray(T, dtype=np.float32)
        w = np.ascontiguousarray(w, dtype=np.float32)
        loss = C.c_double()
        self._c(lib().hf_lc_train_step(self._h, ptr, T.ctypes.data, w.ctypes.data, dt, lr, C.byref(loss)))
        return loss.value

    def stream(self) -> int:
        s = C.c_void_p()
        self._c(lib().hf_lc_stream(self._h, C.byref(s)))
        return s.value or 0

    def features(self):
        """(BF16 bits [nf][64], scale [nf][2]) of the current state: the network's inputs."""
        nf = 2 * self.n * (self.n + 1)
        x = np.empty((nf, 64), np.uint16)
        sc = np.empty((nf, 2), np.float32)
        self._c(lib().hf_lc_features(self._h, x.ctypes.data, sc.ctypes.data))
        return x, sc

    def mlp_forward(self, x_bits: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x_bits, dtype=np.uint16)
        nf = x.shape[0]
        y = np.empty((nf, 4), np.float32)
        self._c(lib().hf_lc_mlp_forward(self._h, x.ctypes.data, nf, y.ctypes.data))
        return y

    def mlp_backward(self, x_bits: np.ndarray, dy: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x_bits, dtype=np.uint16)
        dy = np.ascontiguousarray(dy, dtype=np.float32)
        g = np.empty(NPARAM, np.float32)
        self._c(lib().hf_lc_mlp_backward(self._h, x.ctypes.data, dy.ctypes.data, x.shape[0], g.ctypes.data))
        return g


def _interior(U: np.ndarray, g: int) -> np.ndarray:
    return U[:, g:-g, g:-g]


def fine_pairs(case_fine: dict, t_end: float, factor: int = 4, stride: int = 8):
    """Runs the plain FP64 solver on the fine case until t_end; every `stride`-th window
    of `factor` fine steps gives a pair (filtered state, filtered state after the window,
    summed dt)."""
    s = CartSolver(case_fine)
    g = s.block_dims(0)["ghost"]
    pairs, t, k = [], 0.0, 0
    while t < t_end:
        take = k % stride == 0
        if take:
            U0 = box_filter(_interior(s.state(0), g), factor)
        dtc = 0.0
        for _ in range(factor):
            dtc += s.step()
        if not (dtc > 0.0 and np.isfinite(dtc)):
            s.close()
            raise FloatingPointError(f"fine run stopped advancing at t = {t} (dt = {dtc})")
        if take:
            U1 = box_filter(_interior(s.state(0), g), factor)
            pairs.append((U0.astype(np.float32), U1.astype(np.float32), dtc))
        t += dtc
        k += 1
    s.close()
    return pairs


def fine_sequence(case_fine: dict, t_end: float, factor: int = 4):
    """The plain FP64 solver on the fine case until t_end, box-filtered by `factor` after
    every window of `factor` fine steps: (states [m+1] of [4][n/f][n/f] float32, dts [m])."""
    s = CartSolver(case_fine)
    states = [s.coarsen(0, factor)]
    dts, t = [], 0.0
    while t < t_end:
        dtc = 0.0
        for _ in range(factor):
            dtc += s.step()
        if not (dtc > 0.0 and np.isfinite(dtc)):
            s.close()
            raise FloatingPointError(f"fine run stopped advancing at t = {t} (dt = {dtc})")
        states.append(s.coarsen(0, factor))
        dts.append(dtc)
        t += dtc
    s.close()
    return states, dts


def train_rollout(ls: "LearnedSolver", seqs, iters: int, lr: float = 1e-3, max_roll: int = 4,
                  p_roll: float = 0.5, seed: int = 0, w=None):
    """One-step training on the solver's own inputs ("pushforward"): with probability p_roll
    the input is the learned solver's state after r = 1..max_roll of its own steps from a
    filtered fine state (no gradient through those steps), else the filtered state itself;
    the target is the filtered fine state one window after the input.  seqs: list of
    (states, dts) from fine_sequence."""
    rng = np.random.default_rng(seed)
    if w is None:
        pairs = [(st[k], st[k + 1], dts[k]) for st, dts in seqs for k in range(len(dts))]
        w = change_weights(pairs)
    losses = []
    for it in range(iters):
        st, dts = seqs[int(rng.integers(len(seqs)))]
        r = int(rng.integers(1, max_roll + 1)) if rng.random() < p_roll else 0
        k = int(rng.integers(0, len(dts) - r))
        lr_it = lr * (0.5 * (1 + np.cos(np.pi * it / iters)))
        if r == 0:
            losses.append(ls.train_step(st[k], st[k + 1], w, dts[k], lr_it))
            continue
        ls.set_state(st[k])
        for j in range(r):
            ls.step(dts[k + j], True)
        losses.append(ls.train_step(None, st[k + r + 1], w, dts[k + r], lr_it))
    return np.array(losses), w


def change_weights(pairs) -> np.ndarray:
    """Per-variable loss weights: the inverse mean squared one-step change."""
    acc = np.zeros(4)
    for U0, U1, _ in pairs:
        acc += ((U1.astype(np.float64) - U0) ** 2).mean(axis=(1, 2))
    acc /= len(pairs)
    return (1.0 / (acc + 1e-30)).astype(np.float32)


def train(ls: LearnedSolver, pairs, iters: int, lr: float = 1e-3, seed: int = 0, w=None):
    rng = np.random.default_rng(seed)
    w = change_weights(pairs) if w is None else w
    losses = []
    for it in range(iters):
        U0, T, dt = pairs[int(rng.integers(len(pairs)))]
        lr_it = lr * (0.5 * (1 + np.cos(np.pi * it / iters)))     # cosine decay
        losses.append(ls.train_step(U0, T, w, dt, lr_it))
    return np.array(losses), w


def one_step_loss(ls: LearnedSolver, pairs, w, use_mlp: bool) -> float:
    """Mean weighted one-step error against the filtered fine step (no training)."""
    tot = 0.0
    for U0, T, dt in pairs:
        ls.set_state(U0)
        ls.step(dt, use_mlp)
        U1 = ls.state().astype(np.float64)
        tot += float((w[:, None, None] * (U1 - T) ** 2).mean(axis=(1, 2)).sum())
    return tot / len(pairs)


def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def evaluate_plain(case_fn, n_fine: int, t_end: float, factor: int = 4, limiter: int = 0):
    """L1 density error against the filtered FP64 fine solution, and wall time, of plain FP64
    at n_fine, n_fine/2, n_fine/4 (CartSolver) and plain FP32 at n_fine/4 (LearnedSolver
    without the MLP).  Returns (results, filtered reference density, coarse initial state)."""
    out = {}
    nc = n_fine // factor

    def cart_run(n):
        s = CartSolver(case_fn(n))
        g = s.block_dims(0)["ghost"]
        _, sec = _timed(lambda: s.solve())
        U = _interior(s.state(0), g)
        s.close()
        return U, sec

    Uf, tf = cart_run(n_fine)
    ref = box_filter(Uf, factor)[0]
    out["fp64_fine"] = {"n": n_fine, "seconds": tf, "l1_rho": 0.0}
    for k in (2, 4):
        n = n_fine // k
        U, sec = cart_run(n)
        rho = box_filter(U, factor // k)[0] if factor // k > 1 else U[0]
        out[f"fp64_{n}"] = {"n": n, "seconds": sec, "l1_rho": float(np.abs(rho - ref).mean())}
    # coarse FP32 runs start from the coarse grid's own initial condition
    s0 = CartSolver(case_fn(nc))
    U0 = _interior(s0.state(0), s0.block_dims(0)["ghost"]).astype(np.float32)
    s0.close()
    ls = LearnedSolver(nc, 1.0 / nc, limiter=limiter)
    ls.set_state(U0, 0.0)
    (steps, _), sec = _timed(lambda: ls.run_to(t_end, False))
    rho = ls.state()[0].astype(np.float64)
    out["fp32_plain"] = {"n": nc, "seconds": sec, "steps": steps, "l1_rho": float(np.abs(rho - ref).mean())}
    ls.close()
    return out, ref, U0


def evaluate_learned(t_end: float, params, ref, U0, limiter: int = 0, bound: float | None = None,
                     guard_mode: int = 0) -> dict:
    """The learned FP32 coarse run from U0 to t_end: L1 density error against ref, wall time.
    bound: the change guard's per-cell bound (default: the solver's); guard_mode 1: the
    local-extremum guard instead."""
    nc = U0.shape[1]
    ls = LearnedSolver(nc, 1.0 / nc, limiter=limiter)
    ls.set_params(params)
    if bound is not None:
        ls.set_bound(bound)
    ls.set_guard_mode(guard_mode)
    ls.set_state(U0, 0.0)
    (steps, rej), sec = _timed(lambda: ls.run_to(t_end, True))
    rho = ls.state()[0].astype(np.float64)
    ls.close()
    return {"n": nc, "seconds": sec, "steps": steps, "rejected_cells": rej,
            "l1_rho": float(np.abs(rho - ref).mean())}


def evaluate(case_fn, n_fine: int, t_end: float, params, factor: int = 4, limiter: int = 0):
    """evaluate_plain plus the learned run (key fp32_learned)."""
    out, ref, U0 = evaluate_plain(case_fn, n_fine, t_end, factor, limiter)
    out["fp32_learned"] = evaluate_learned(t_end, params, ref, U0, limiter)
    return out
