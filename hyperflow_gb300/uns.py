"""Python host mirror of the reference's unstructured solver (src/fvm_2d_uns).

``UnsSolver`` runs the reference's unstructured step -- TimeStep (timestep.cpp:29-62),
GodunovScheme + forward Euler (godunov.cpp:31-77) -- on the GPU through the C ABI of
include/hyperflow_gb300_uns.h.  Meshes use the reference's text format, extended to
triangles (see meshgen.py).
"""
from __future__ import annotations

import ctypes as C
import json
import warnings

import numpy as np

from ._lib import check, lib

_MSG = "hf_uns_last_error_message"


class MeshWarning(UserWarning):
    """A mesh loaded with interior pairs that have no partner edge."""


def mesh_neighbours(mesh: str | bytes):
    """The loader's neighbour search alone, on the host (no GPU): (nbr per pair, unmatched
    count, first unmatched pair or -1) for a mesh in the text or binary format."""
    raw = mesh if isinstance(mesh, bytes) else mesh.encode()
    L = lib()
    nc, npair, un, first = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    check(L.hf_uns_mesh_neighbours(raw, len(raw), C.byref(nc), C.byref(npair), None, 0, None, None))
    nbr = np.empty(npair.value, np.int32)
    check(L.hf_uns_mesh_neighbours(raw, len(raw), C.byref(nc), C.byref(npair), nbr.ctypes.data, nbr.size,
                                   C.byref(un), C.byref(first)))
    return nbr, un.value, first.value


class UnsSolver:
    def __init__(self, case, mesh_text: str | bytes | None = None):
        """mesh_text: the mesh in memory instead of the case's mesh.file -- the text format
        (str) or the binary format's bytes (``meshgen.hmshb_bytes``); a mesh.file may hold
        either, told apart by the binary format's magic."""
        text = case if isinstance(case, str) else json.dumps(case)
        self.case = json.loads(text)
        raw = text.encode()
        L = lib()
        h = C.c_void_p()
        if mesh_text is None:
            st = L.hf_uns_create(raw, len(raw), C.byref(h))
        else:
            mt = mesh_text if isinstance(mesh_text, bytes) else mesh_text.encode()
            st = L.hf_uns_create_mesh(raw, len(raw), mt, len(mt), C.byref(h))
        self._h = h
        if st != 0:
            try:
                check(st, h, _MSG)
            finally:
                if h:
                    L.hf_uns_destroy(h)
                self._h = None
        nc, npair = C.c_int64(), C.c_int64()
        check(L.hf_uns_sizes(self._h, C.byref(nc), C.byref(npair)), self._h, _MSG)
        self.ncells, self.npairs = nc.value, npair.value
        n_unmatched, first = self.unmatched_pairs()
        if n_unmatched:
            warnings.warn(f"mesh: {n_unmatched} interior (cell-coded) pairs match no edge within 1e-12 and "
                          f"take their code as the neighbour cell, as the reference does (first: pair {first})",
                          MeshWarning, stacklevel=2)

    def close(self):
        if getattr(self, "_h", None):
            lib().hf_uns_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def unmatched_pairs(self):
        """(count, first pair index or -1) of the pairs whose code names a cell (0: an interior
        edge) but that found no partner; they take the code as their neighbour, as in the
        reference's loader."""
        n, first = C.c_int64(), C.c_int64()
        check(lib().hf_uns_unmatched_pairs(self._h, C.byref(n), C.byref(first)), self._h, _MSG)
        return n.value, first.value

    def mesh_arrays(self):
        ps = np.empty(self.ncells + 1, np.int32)
        nbr = np.empty(self.npairs, np.int32)
        ang, ln = np.empty(self.npairs), np.empty(self.npairs)
        area, rin = np.empty(self.ncells), np.empty(self.ncells)
        check(lib().hf_uns_mesh_arrays(self._h, ps.ctypes.data, nbr.ctypes.data, ang.ctypes.data,
                                       ln.ctypes.data, area.ctypes.data, rin.ctypes.data), self._h, _MSG)
        return {"pair_start": ps, "nbr": nbr, "angle": ang, "length": ln, "area": area, "rin": rin}

    def state(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((4, self.ncells))
        check(lib().hf_uns_get_state(self._h, out.ctypes.data), self._h, _MSG)
        return out

    def set_state(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.shape == (4, self.ncells)
        check(lib().hf_uns_set_state(self._h, U.ctypes.data), self._h, _MSG)

    def calculate_time_step(self) -> float:
        dt = C.c_double()
        check(lib().hf_uns_time_step(self._h, C.byref(dt)), self._h, _MSG)
        return dt.value

    def advance(self, dt: float):
        check(lib().hf_uns_advance(self._h, dt), self._h, _MSG)

    def run(self, n: int, clamp_t_end: bool = False, graph: bool = True) -> int:
        done = C.c_int64()
        check(lib().hf_uns_run(self._h, n, int(clamp_t_end), int(graph), C.byref(done)), self._h, _MSG)
        return done.value

    def time(self):
        t, c, d = C.c_double(), C.c_int64(), C.c_double()
        check(lib().hf_uns_get_time(self._h, C.byref(t), C.byref(c), C.byref(d)), self._h, _MSG)
        return t.value, c.value, d.value

    def hllc_errors(self) -> int:
        n = C.c_int64()
        check(lib().hf_uns_hllc_errors(self._h, C.byref(n)), self._h, _MSG)
        return n.value

    def set_edge_mode(self, edge_based: bool):
        """False: per-(cell, edge) fluxes, bit-identical to the reference (default).
        True: one flux per unique interior edge (half the HLLC work)."""
        check(lib().hf_uns_set_edge_mode(self._h, int(edge_based)), self._h, _MSG)

    def centroids(self) -> np.ndarray:
        """[2][ncells] cell centroids as the reference computes them"""
        out = np.empty((2, self.ncells))
        check(lib().hf_uns_centroids(self._h, out.ctypes.data), self._h, _MSG)
        return out

    # --- frames (Simulation::solve's output cadence, captured on the device) ---
    def enable_frames(self, ring_slots: int = 8):
        check(lib().hf_uns_frames_enable(self._h, ring_slots), self._h, _MSG)

    def frames_pending(self) -> int:
        n = C.c_int64()
        check(lib().hf_uns_frames_pending(self._h, C.byref(n)), self._h, _MSG)
        return n.value

    def pop_frame(self):
        """(frame index, time label, cell states [4][ncells])"""
        buf = np.empty((4, self.ncells))
        t, idx = C.c_double(), C.c_int64()
        check(lib().hf_uns_frame_pop(self._h, buf.ctypes.data, C.byref(t), C.byref(idx)), self._h, _MSG)
        return idx.value, t.value, buf

    def solve(self, out_dir: str | None = None, fmt: str = "hfb", ring_slots: int = 8,
              chunk: int = 1000) -> int:
        """Runs to t_end like the unstructured Simulation::solve (simulation.cpp:51-120);
        with out_dir, also its frame dt clamp and output cadence, frames written as
        results_%06d.hfb (binary) or, with fmt="csv", the reference's own CSV text."""
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
        meta = frames.uns_case_meta(self.case, self.ncells)
        self.enable_frames(ring_slots)
        writer = frames.FrameWriter(out_dir, meta, fmt, centroids=self.centroids())
        total, next_index = 0, 0
        try:
            while True:
                k = self.run(chunk, clamp_t_end=True)
                total += k
                popped = 0
                while self.frames_pending() > 0:
                    idx, t, U = self.pop_frame()
                    writer.put(idx, t, [U])
                    next_index = idx + 1
                    popped += 1
                t_now = self.time()[0]
                if t_now == meta["t_end"]:
                    break
                if k == 0 and popped == 0:
                    raise RuntimeError("device loop made no progress before t_end")
            writer.put(next_index, t_now, [self.state()])
        finally:
            paths = writer.close()
            self.enable_frames(0)
        self.frame_paths = paths
        return total

    def sync(self):
        """Waits for the solver's stream; raises if a kernel raised the device error word."""
        check(lib().hf_uns_sync(self._h), self._h, _MSG)

    def set_strict(self, on: bool = True):
        """Strict mode: a zero-flux HLLC pair or a cell left with a non-positive density or
        pressure stops the loop and raises HyperFlowError."""
        check(lib().hf_uns_set_strict(self._h, int(bool(on))), self._h, _MSG)

    def last_error_cell(self):
        """The earliest zero-flux (cell, pair): dict(step, cell), or None."""
        cell, st = C.c_int64(), C.c_int64()
        check(lib().hf_uns_last_error_cell(self._h, C.byref(cell), C.byref(st)), self._h, _MSG)
        return None if cell.value < 0 else {"step": st.value, "cell": cell.value}

    def last_nonpositive_cell(self):
        """The earliest cell a step left with density or pressure not positive (zero, negative
        or NaN): dict(step, cell), or None."""
        cell, st = C.c_int64(), C.c_int64()
        check(lib().hf_uns_last_nonpositive_cell(self._h, C.byref(cell), C.byref(st)), self._h, _MSG)
        return None if cell.value < 0 else {"step": st.value, "cell": cell.value}

    def clear_error_cell(self):
        """Forgets both records (zero-flux pair and non-positive cell)."""
        check(lib().hf_uns_clear_error_cell(self._h), self._h, _MSG)

    # --- checkpoint / restart ---
    def checkpoint(self) -> bytes:
        """The whole simulation state as bytes; ``restore`` on a solver of the same case and
        mesh continues bit for bit."""
        n = C.c_size_t()
        check(lib().hf_uns_checkpoint_size(self._h, C.byref(n)), self._h, _MSG)
        buf = np.empty(n.value, np.uint8)
        check(lib().hf_uns_checkpoint_save(self._h, buf.ctypes.data, n.value), self._h, _MSG)
        return buf.tobytes()

    def restore(self, blob: bytes):
        buf = np.frombuffer(blob, np.uint8)
        check(lib().hf_uns_checkpoint_load(self._h, buf.ctypes.data, buf.size), self._h, _MSG)

    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().hf_uns_stream(self._h, C.byref(s)), self._h, _MSG)
        return s.value or 0
