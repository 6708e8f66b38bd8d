"""Python host mirror of the reference's Cartesian solver interface.

``CartSolver`` exposes the reference's step pieces under their own names
(src/fvm_2d_cart): ``apply_bcs`` (Mesh::apply_bcs, mesh.cpp:31-39),
``calculate_time_step`` (Scheme::calculate_time_step -> TimeStep::operator(),
timestep.cpp:29-68), ``advance_block`` / ``advance`` (ODESolver(Scheme(block)) +
set_fields, simulation.cpp:106-110), and ``solve``-style loops (simulation.cpp:51-124)
-- all executed by the CUDA kernels behind the C ABI of include/hyperflow_gb300.h.
"""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from ._lib import LAYOUT_AOS_XY, LAYOUT_SOA, check, lib


class CartSolver:
    """One case file -> one device-resident simulation (FP64 SoA state in HBM)."""

    def __init__(self, case):
        text = case if isinstance(case, str) else json.dumps(case)
        self.case = json.loads(text)
        raw = text.encode()
        L = lib()
        h = C.c_void_p()
        st = L.hf_create(raw, len(raw), C.byref(h))
        self._h = h
        if st != 0:
            try:
                check(st, h)
            finally:
                if h:
                    L.hf_destroy(h)
                self._h = None
        n = C.c_int()
        check(L.hf_num_blocks(self._h, C.byref(n)), self._h)
        self.nblocks = n.value

    # --- lifecycle ---
    def close(self):
        if getattr(self, "_h", None):
            lib().hf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- geometry ---
    def block_dims(self, b: int = 0) -> dict:
        d = (C.c_int * 5)()
        check(lib().hf_block_dims(self._h, b, d), self._h)
        return {"total_x": d[0], "total_y": d[1], "ghost": d[2], "x_cells": d[3], "y_cells": d[4]}

    def interior_cells(self) -> int:
        return sum(self.block_dims(b)["x_cells"] * self.block_dims(b)["y_cells"]
                   for b in range(self.nblocks))

    # --- state ---
    def state(self, b: int = 0, layout: str = "soa", out: np.ndarray | None = None) -> np.ndarray:
        """SoA [var][y][x] (default) or MeshBlock order [x][y][var], ghosts included.
        ``out`` (SoA, C-contiguous float64, e.g. pinned memory) receives the copy."""
        d = self.block_dims(b)
        if layout == "soa":
            if out is None:
                out = np.empty((4, d["total_y"], d["total_x"]))
            assert out.shape == (4, d["total_y"], d["total_x"]) and out.flags.c_contiguous
            check(lib().hf_get_state(self._h, b, out.ctypes.data, LAYOUT_SOA), self._h)
        else:
            out = np.empty((d["total_x"], d["total_y"], 4))
            check(lib().hf_get_state(self._h, b, out.ctypes.data, LAYOUT_AOS_XY), self._h)
        return out

    def set_state(self, b: int, U: np.ndarray, layout: str = "soa"):
        U = np.ascontiguousarray(U, dtype=np.float64)
        lay = LAYOUT_SOA if layout == "soa" else LAYOUT_AOS_XY
        check(lib().hf_set_state(self._h, b, U.ctypes.data, lay), self._h)

    # --- the reference's step pieces ---
    def apply_bcs(self):
        check(lib().hf_apply_bcs(self._h), self._h)

    def calculate_time_step(self) -> float:
        dt = C.c_double()
        check(lib().hf_time_step(self._h, C.byref(dt)), self._h)
        return dt.value

    def advance_block(self, b: int, dt: float):
        check(lib().hf_advance_block(self._h, b, dt), self._h)

    def advance(self, dt: float):
        check(lib().hf_advance(self._h, dt), self._h)

    def step(self) -> float:
        dt = C.c_double()
        check(lib().hf_step(self._h, C.byref(dt)), self._h)
        return dt.value

    def step_io(self, ins, outs=None) -> float:
        """One step with every block's state in host arrays (SoA [4][total_y][total_x], ghosts
        included, C-contiguous float64): upload, step, download into outs (default: in place).
        Pinned arrays (``host_mapped``) are read and written by the kernels directly; others
        are copied.  Returns the step's dt."""
        outs = ins if outs is None else outs
        assert len(ins) == len(outs) == self.nblocks
        for a in list(ins) + list(outs):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        pin = (C.c_void_p * self.nblocks)(*[a.ctypes.data for a in ins])
        pout = (C.c_void_p * self.nblocks)(*[a.ctypes.data for a in outs])
        dt = C.c_double()
        check(lib().hf_step_io(self._h, pin, pout, C.byref(dt)), self._h)
        return dt.value

    @staticmethod
    def host_mapped(a: np.ndarray) -> bool:
        """True when the kernels address this host array directly (pinned memory)."""
        m = C.c_int()
        check(lib().hf_host_mapped(a.ctypes.data, C.byref(m)))
        return bool(m.value)

    def run(self, n: int, clamp_t_end: bool = False, graph: bool = True) -> int:
        done = C.c_int64()
        check(lib().hf_run(self._h, n, int(clamp_t_end), int(graph), C.byref(done)), self._h)
        return done.value

    def solve(self, out_dir: str | None = None, fmt: str = "hfb", ring_slots: int = 8,
              chunk: int = 1000) -> int:
        """Runs to t_end like Simulation::solve (simulation.cpp:51-124); returns steps taken.

        Without out_dir: the t_end clamp only (no frame clamp, no output).  With out_dir: the
        reference's frame dt clamp and output cadence as well (the case's
        simulation.animation), frames captured on the device and written by a background
        thread as results_%06d.hfb (binary, full precision; ``frames.read_frame``) or, with
        fmt="csv", as the reference's own results_%06d.csv text."""
        if out_dir is None:
            total = 0
            while True:
                t0 = self.time()[0]
                k = self.run(chunk, clamp_t_end=True)
                total += k
                if k < chunk:
                    return total
                if not self.time()[0] > t0:
                    raise FloatingPointError(f"time stopped advancing at t = {t0} (dt = 0 or NaN)")
        from . import frames
        meta = frames.case_meta(self.case)
        self.enable_frames(ring_slots)
        writer = frames.FrameWriter(out_dir, meta, fmt)
        total, next_index = 0, 0
        try:
            while True:
                k = self.run(chunk, clamp_t_end=True)
                total += k
                popped = 0
                while self.frames_pending() > 0:
                    idx, t, blocks = self.pop_frame()
                    writer.put(idx, t, blocks)
                    next_index = idx + 1
                    popped += 1
                t_now = self.time()[0]
                if t_now == meta["t_end"]:
                    break
                if k == 0 and popped == 0:
                    raise RuntimeError("device loop made no progress before t_end")
            g = self.block_dims(0)["ghost"]
            writer.put(next_index, t_now, [self.state(b)[:, g:-g, g:-g].copy() for b in range(self.nblocks)])
        finally:
            paths = writer.close()
            self.enable_frames(0)
        self.frame_paths = paths
        return total

    # --- frames (Simulation::solve's output cadence, captured on the device) ---
    def enable_frames(self, ring_slots: int = 8):
        check(lib().hf_frames_enable(self._h, ring_slots), self._h)

    def frames_pending(self) -> int:
        n = C.c_int64()
        check(lib().hf_frames_pending(self._h, C.byref(n)), self._h)
        return n.value

    def pop_frame(self):
        """(frame index, time label, per-block interior states [4][ny][nx])"""
        n = C.c_int64()
        check(lib().hf_frame_len(self._h, C.byref(n)), self._h)
        buf = np.empty(n.value)
        t, idx = C.c_double(), C.c_int64()
        check(lib().hf_frame_pop(self._h, buf.ctypes.data, C.byref(t), C.byref(idx)), self._h)
        blocks, o = [], 0
        for b in range(self.nblocks):
            d = self.block_dims(b)
            m = 4 * d["x_cells"] * d["y_cells"]
            blocks.append(buf[o:o + m].reshape(4, d["y_cells"], d["x_cells"]))
            o += m
        return idx.value, t.value, blocks

    def coarsen(self, b: int = 0, factor: int = 4) -> np.ndarray:
        """factor x factor box average of block b's interior, FP32 [4][ny/f][nx/f], formed
        on the device."""
        d = self.block_dims(b)
        out = np.empty((4, d["y_cells"] // factor, d["x_cells"] // factor), np.float32)
        check(lib().hf_coarsen(self._h, b, factor, out.ctypes.data), self._h)
        return out

    # --- checkpoint / restart ---
    def checkpoint(self) -> bytes:
        """The whole simulation state (both state buffers, ghosts, t, call count, frame
        cadence) as bytes; ``restore`` on a solver of the same case continues bit for bit."""
        n = C.c_size_t()
        check(lib().hf_checkpoint_size(self._h, C.byref(n)), self._h)
        buf = np.empty(n.value, np.uint8)
        check(lib().hf_checkpoint_save(self._h, buf.ctypes.data, n.value), self._h)
        return buf.tobytes()

    def restore(self, blob: bytes):
        buf = np.frombuffer(blob, np.uint8)
        check(lib().hf_checkpoint_load(self._h, buf.ctypes.data, buf.size), self._h)

    def save_checkpoint(self, path: str):
        with open(path, "wb") as fh:
            fh.write(self.checkpoint())

    def load_checkpoint(self, path: str):
        with open(path, "rb") as fh:
            self.restore(fh.read())

    def sync(self):
        check(lib().hf_sync(self._h), self._h)

    # --- introspection ---
    def time(self):
        t, c, d = C.c_double(), C.c_int64(), C.c_double()
        check(lib().hf_get_time(self._h, C.byref(t), C.byref(c), C.byref(d)), self._h)
        return t.value, c.value, d.value

    def hllc_errors(self) -> int:
        n = C.c_int64()
        check(lib().hf_hllc_errors(self._h, C.byref(n)), self._h)
        return n.value

    def set_strict(self, on: bool = True):
        """Strict mode: a zero-flux HLLC face or a cell left with a non-positive density or
        pressure stops the loop and raises HyperFlowError (HF_ERR_NUMERIC); off (the default)
        the run continues as the reference's does."""
        check(lib().hf_set_strict(self._h, int(bool(on))), self._h)

    def last_error_cell(self):
        """The earliest zero-flux face: dict(step, block, dir, i, j), or None."""
        v = [C.c_int() for _ in range(4)]
        st = C.c_int64()
        check(lib().hf_last_error_cell(self._h, *[C.byref(x) for x in v], C.byref(st)), self._h)
        if v[0].value < 0:
            return None
        return {"step": st.value, "block": v[0].value, "i": v[1].value, "j": v[2].value, "dir": v[3].value}

    def last_nonpositive_cell(self):
        """The earliest interior cell a step left with density or pressure not positive (zero,
        negative or NaN): dict(step, block, i, j), or None."""
        v = [C.c_int() for _ in range(3)]
        st = C.c_int64()
        check(lib().hf_last_nonpositive_cell(self._h, *[C.byref(x) for x in v], C.byref(st)), self._h)
        if v[0].value < 0:
            return None
        return {"step": st.value, "block": v[0].value, "i": v[1].value, "j": v[2].value}

    def clear_error_cell(self):
        """Forgets both records (zero-flux face and non-positive cell)."""
        check(lib().hf_clear_error_cell(self._h), self._h)

    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().hf_stream(self._h, C.byref(s)), self._h)
        return s.value or 0

    def set_block_launches(self, per_block: bool):
        """True: one stencil launch per block, in order.  False (default): a MUSCL-Hancock step
        of up to 4 blocks is one launch that checks each block's predictor dt against the
        reference's and runs a block again where it differs; the results are identical."""
        check(lib().hf_set_block_launches(self._h, int(bool(per_block))), self._h)

    def blocks_rerun(self) -> int:
        """block updates run a second time because their predictor dt changed (all-blocks launch)"""
        n = C.c_int64()
        check(lib().hf_blocks_rerun(self._h, C.byref(n)), self._h)
        return n.value

    def profile(self, enable: bool = True):
        check(lib().hf_profile(self._h, int(enable)), self._h)

    def kernel_time(self, kind: int = 0):
        ms, n = C.c_double(), C.c_int64()
        check(lib().hf_kernel_time(self._h, kind, C.byref(ms), C.byref(n)), self._h)
        return ms.value, n.value
