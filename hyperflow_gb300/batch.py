"""Python host mirror of the batched MUSCL-Hancock entry points
(include/hyperflow_gb300_batch.h): many independent single-block cases, one persistent
cooperative kernel per run of steps, optional CUDA graph, autotuned launch shape."""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from ._lib import check, lib

_MSG = "hf_batch_last_error_message"


def configs():
    n = C.c_int()
    check(lib().hf_batch_num_configs(C.byref(n)))
    out = []
    for k in range(n.value):
        v = [C.c_int() for _ in range(4)]
        check(lib().hf_batch_config_info(k, *[C.byref(x) for x in v]))
        out.append({"tile_x": v[0].value, "tile_y": v[1].value, "threads": v[2].value,
                    "stages": v[3].value})
    return out


class BatchSolver:
    def __init__(self, manifest):
        text = manifest if isinstance(manifest, str) else json.dumps(manifest)
        raw = text.encode()
        L = lib()
        h = C.c_void_p()
        st = L.hf_batch_create(raw, len(raw), C.byref(h))
        self._h = h
        if st != 0:
            try:
                check(st, h, _MSG)
            finally:
                if h:
                    L.hf_batch_destroy(h)
                self._h = None
        n, cells = C.c_int(), C.c_int64()
        check(L.hf_batch_sizes(self._h, C.byref(n), C.byref(cells)), self._h, _MSG)
        self.ninstances, self.total_cells = n.value, cells.value
        self.sides = []
        for i in range(self.ninstances):
            s = C.c_int()
            check(L.hf_batch_instance_side(self._h, i, C.byref(s)), self._h, _MSG)
            self.sides.append(s.value)

    def close(self):
        if getattr(self, "_h", None):
            lib().hf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_config(self, k: int):
        check(lib().hf_batch_set_config(self._h, k), self._h, _MSG)

    def autotune(self, steps_per_trial: int = 2):
        best = C.c_int()
        n = len(configs())
        ms = np.zeros(n)
        check(lib().hf_batch_autotune(self._h, steps_per_trial, C.byref(best), ms.ctypes.data),
              self._h, _MSG)
        return best.value, ms

    def run(self, nsteps: int, graph: bool = True):
        check(lib().hf_batch_run(self._h, nsteps, int(graph)), self._h, _MSG)

    def sync(self):
        check(lib().hf_batch_sync(self._h), self._h, _MSG)

    def state(self, i: int) -> np.ndarray:
        n = self.sides[i]
        out = np.empty((4, n, n))
        check(lib().hf_batch_get_state(self._h, i, out.ctypes.data), self._h, _MSG)
        return out

    def set_state(self, i: int, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        check(lib().hf_batch_set_state(self._h, i, U.ctypes.data), self._h, _MSG)

    def instance_time(self, i: int):
        t, d = C.c_double(), C.c_double()
        check(lib().hf_batch_instance_time(self._h, i, C.byref(t), C.byref(d)), self._h, _MSG)
        return t.value, d.value

    def counters(self):
        s, c, e = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().hf_batch_counters(self._h, C.byref(s), C.byref(c), C.byref(e)), self._h, _MSG)
        return {"steps": s.value, "calls": c.value, "hllc_errors": e.value}

    def last_nonpositive_cell(self):
        """The earliest cell a step left with density or pressure not positive (zero, negative
        or NaN): dict(step, case, i, j), or None."""
        v = [C.c_int() for _ in range(3)]
        st = C.c_int64()
        check(lib().hf_batch_last_nonpositive_cell(self._h, *[C.byref(x) for x in v], C.byref(st)),
              self._h, _MSG)
        if v[0].value < 0:
            return None
        return {"step": st.value, "case": v[0].value, "i": v[1].value, "j": v[2].value}

    def clear_error_cell(self):
        check(lib().hf_batch_clear_error_cell(self._h), self._h, _MSG)

    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().hf_batch_stream(self._h, C.byref(s)), self._h, _MSG)
        return s.value or 0
