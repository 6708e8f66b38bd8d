"""Loads the in-tree CUDA library and declares the C-ABI signatures.

There is no CPU fallback: if ``libhyperflow_gb300.so`` is missing, or a call needs
a GPU and none is visible, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
# HF_LIB_VARIANT=checked loads the bounds-checked build (libhyperflow_gb300_checked.so, made by
# _build.build(variant="checked")): same results, and an out-of-range index sets the error word
_VARIANT = os.environ.get("HF_LIB_VARIANT", "")
LIB_PATH = os.path.join(PKG, "libhyperflow_gb300%s.so" % ("_" + _VARIANT if _VARIANT else ""))

HF_OK = 0
STATUS = {0: "ok", 1: "bad argument", 2: "case file parse error", 3: "unsupported case",
          4: "CUDA error", 5: "device error word raised", 6: "call out of order",
          7: "no CUDA device", 8: "problem exceeds the fixed-size working area",
          9: "strict mode: an HLLC zero-flux fallback or a non-positive density or pressure occurred"}

LAYOUT_SOA = 0
LAYOUT_AOS_XY = 1

# every symbol include/hyperflow_gb300.h declares: name -> (restype, argtypes)
_p, _i, _d, _sz, _i64 = C.c_void_p, C.c_int, C.c_double, C.c_size_t, C.c_int64
SIGNATURES = {
    "hf_create": (_i, [C.c_char_p, _sz, C.POINTER(_p)]),
    "hf_destroy": (None, [_p]),
    "hf_num_blocks": (_i, [_p, C.POINTER(_i)]),
    "hf_block_dims": (_i, [_p, _i, C.POINTER(_i)]),
    "hf_set_state": (_i, [_p, _i, _p, _i]),
    "hf_get_state": (_i, [_p, _i, _p, _i]),
    "hf_apply_bcs": (_i, [_p]),
    "hf_time_step": (_i, [_p, C.POINTER(_d)]),
    "hf_advance_block": (_i, [_p, _i, _d]),
    "hf_advance": (_i, [_p, _d]),
    "hf_step": (_i, [_p, C.POINTER(_d)]),
    "hf_step_io": (_i, [_p, _p, _p, C.POINTER(_d)]),
    "hf_host_mapped": (_i, [_p, C.POINTER(_i)]),
    "hf_set_strict": (_i, [_p, _i]),
    "hf_last_error_cell": (_i, [_p, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i64)]),
    "hf_last_nonpositive_cell": (_i, [_p, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i64)]),
    "hf_clear_error_cell": (_i, [_p]),
    "hf_run": (_i, [_p, _i64, _i, _i, C.POINTER(_i64)]),
    "hf_get_time": (_i, [_p, C.POINTER(_d), C.POINTER(_i64), C.POINTER(_d)]),
    "hf_hllc_errors": (_i, [_p, C.POINTER(_i64)]),
    "hf_sync": (_i, [_p]),
    "hf_stream": (_i, [_p, C.POINTER(_p)]),
    "hf_profile": (_i, [_p, _i]),
    "hf_kernel_time": (_i, [_p, _i, C.POINTER(_d), C.POINTER(_i64)]),
    "hf_frames_enable": (_i, [_p, _i]),
    "hf_frame_len": (_i, [_p, C.POINTER(_i64)]),
    "hf_frames_pending": (_i, [_p, C.POINTER(_i64)]),
    "hf_frame_pop": (_i, [_p, _p, C.POINTER(_d), C.POINTER(_i64)]),
    "hf_coarsen": (_i, [_p, _i, _i, _p]),
    "hf_checkpoint_size": (_i, [_p, C.POINTER(_sz)]),
    "hf_checkpoint_save": (_i, [_p, _p, _sz]),
    "hf_checkpoint_load": (_i, [_p, _p, _sz]),
    "hf_status_string": (C.c_char_p, [_i]),
    "hf_set_block_launches": (_i, [_p, _i]),
    "hf_blocks_rerun": (_i, [_p, C.POINTER(_i64)]),
    "hf_time_step_noalloc": (_i, [_p, _i, _i, _i, _d, _d, _d, _d, _i64, _p, _p]),
    # unstructured (include/hyperflow_gb300_uns.h)
    "hf_uns_create": (_i, [C.c_char_p, _sz, C.POINTER(_p)]),
    "hf_uns_create_mesh": (_i, [C.c_char_p, _sz, C.c_char_p, _sz, C.POINTER(_p)]),
    "hf_uns_destroy": (None, [_p]),
    "hf_uns_last_error_message": (C.c_char_p, [_p]),
    "hf_uns_sizes": (_i, [_p, C.POINTER(_i64), C.POINTER(_i64)]),
    "hf_uns_mesh_arrays": (_i, [_p, _p, _p, _p, _p, _p, _p]),
    "hf_uns_unmatched_pairs": (_i, [_p, C.POINTER(_i64), C.POINTER(_i64)]),
    "hf_uns_mesh_neighbours": (_i, [C.c_char_p, _sz, C.POINTER(_i64), C.POINTER(_i64), _p, _i64,
                                    C.POINTER(_i64), C.POINTER(_i64)]),
    "hf_uns_set_state": (_i, [_p, _p]),
    "hf_uns_get_state": (_i, [_p, _p]),
    "hf_uns_time_step": (_i, [_p, C.POINTER(_d)]),
    "hf_uns_advance": (_i, [_p, _d]),
    "hf_uns_run": (_i, [_p, _i64, _i, _i, C.POINTER(_i64)]),
    "hf_uns_centroids": (_i, [_p, _p]),
    "hf_uns_frames_enable": (_i, [_p, _i]),
    "hf_uns_frames_pending": (_i, [_p, C.POINTER(_i64)]),
    "hf_uns_frame_pop": (_i, [_p, _p, C.POINTER(_d), C.POINTER(_i64)]),
    "hf_uns_sync": (_i, [_p]),
    "hf_uns_set_strict": (_i, [_p, _i]),
    "hf_uns_last_error_cell": (_i, [_p, C.POINTER(_i64), C.POINTER(_i64)]),
    "hf_uns_last_nonpositive_cell": (_i, [_p, C.POINTER(_i64), C.POINTER(_i64)]),
    "hf_uns_clear_error_cell": (_i, [_p]),
    "hf_uns_checkpoint_size": (_i, [_p, C.POINTER(_sz)]),
    "hf_uns_checkpoint_save": (_i, [_p, _p, _sz]),
    "hf_uns_checkpoint_load": (_i, [_p, _p, _sz]),
    "hf_uns_get_time": (_i, [_p, C.POINTER(_d), C.POINTER(_i64), C.POINTER(_d)]),
    "hf_uns_hllc_errors": (_i, [_p, C.POINTER(_i64)]),
    "hf_uns_stream": (_i, [_p, C.POINTER(_p)]),
    "hf_uns_set_edge_mode": (_i, [_p, _i]),
    "hf_last_error_message": (C.c_char_p, [_p]),
    # batched (include/hyperflow_gb300_batch.h)
    "hf_batch_create": (_i, [C.c_char_p, _sz, C.POINTER(_p)]),
    "hf_batch_destroy": (None, [_p]),
    "hf_batch_last_error_message": (C.c_char_p, [_p]),
    "hf_batch_sizes": (_i, [_p, C.POINTER(_i), C.POINTER(_i64)]),
    "hf_batch_instance_side": (_i, [_p, _i, C.POINTER(_i)]),
    "hf_batch_num_configs": (_i, [C.POINTER(_i)]),
    "hf_batch_config_info": (_i, [_i, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    "hf_batch_set_config": (_i, [_p, _i]),
    "hf_batch_autotune": (_i, [_p, _i, C.POINTER(_i), _p]),
    "hf_batch_run": (_i, [_p, _i64, _i]),
    "hf_batch_sync": (_i, [_p]),
    "hf_batch_get_state": (_i, [_p, _i, _p]),
    "hf_batch_set_state": (_i, [_p, _i, _p]),
    "hf_batch_instance_time": (_i, [_p, _i, C.POINTER(_d), C.POINTER(_d)]),
    "hf_batch_counters": (_i, [_p, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64)]),
    "hf_batch_last_nonpositive_cell": (_i, [_p, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i64)]),
    "hf_batch_clear_error_cell": (_i, [_p]),
    "hf_batch_stream": (_i, [_p, C.POINTER(_p)]),
    # learned coarse solver (include/hyperflow_gb300_learned.h)
    "hf_lc_create": (_i, [_i, _d, _d, _d, _i, C.POINTER(_p)]),
    "hf_lc_destroy": (None, [_p]),
    "hf_lc_last_error_message": (C.c_char_p, [_p]),
    "hf_lc_num_params": (_i, [C.POINTER(_i)]),
    "hf_lc_set_params": (_i, [_p, _p]),
    "hf_lc_get_params": (_i, [_p, _p]),
    "hf_lc_set_bound": (_i, [_p, _d]),
    "hf_lc_set_guard_mode": (_i, [_p, _i]),
    "hf_lc_set_train_guard": (_i, [_p, _i]),
    "hf_lc_set_fused": (_i, [_p, _i, _i]),
    "hf_lc_set_state": (_i, [_p, _p]),
    "hf_lc_get_state": (_i, [_p, _p]),
    "hf_lc_set_time": (_i, [_p, _d]),
    "hf_lc_get_time": (_i, [_p, C.POINTER(_d)]),
    "hf_lc_cfl_dt": (_i, [_p, C.POINTER(_d)]),
    "hf_lc_step": (_i, [_p, _d, _i, C.POINTER(_i64)]),
    "hf_lc_run_to": (_i, [_p, _d, _i, C.POINTER(_i64), C.POINTER(_i64)]),
    "hf_lc_train_step": (_i, [_p, _p, _p, _p, _d, _d, C.POINTER(_d)]),
    "hf_lc_features": (_i, [_p, _p, _p]),
    "hf_lc_mlp_forward": (_i, [_p, _p, _i, _p]),
    "hf_lc_mlp_backward": (_i, [_p, _p, _p, _i, _p]),
    "hf_lc_stream": (_i, [_p, C.POINTER(_p)]),
    # self-tests (include/hyperflow_gb300_diag.h)
    "hf_render_gray": (_i, [_p, _i, _i, _d, _d, _i, _d, _d, _p, _p, _p, _p]),
    "hf_diag_div_check": (_i, [C.c_uint64, _i64, _i, C.POINTER(_i64), _p]),
}

_lib = None


class HyperFlowError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}" if msg else STATUS.get(status, str(status)))


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, ctx=None, msgfn: str = "hf_last_error_message") -> None:
    if status != HF_OK:
        msg = ""
        if ctx is not None:
            m = getattr(lib(), msgfn)(ctx)
            msg = m.decode() if m else ""
        raise HyperFlowError(status, msg)
