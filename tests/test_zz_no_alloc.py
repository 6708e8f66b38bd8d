"""The no-allocation CFL entry point, hf_time_step_noalloc.

It exists for callers that cannot call cudaMalloc (applications that give all device
memory to their own pool, or time loops under a no-allocation rule): it takes the state
and the output word in the caller's device memory and works in a fixed static device
array.  It must give the same dt as the context-based hf_time_step, bit for bit, call
after call -- including after a larger call has left partial results in the shared
array.  This file is collected last so that a failure here stops a -x run only after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_copy(U):
    import torch
    return torch.from_numpy(np.ascontiguousarray(U)).cuda()


def _noalloc_dt(L, d_state, tx, ty, dx, dy, call_index, cfl=0.8):
    import torch
    d_dt = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = L.hf_time_step_noalloc(d_state.data_ptr(), tx, ty, tx, dx, dy, 1.4, cfl, call_index,
                                d_dt.data_ptr(), None)
    assert st == 0, st
    torch.cuda.synchronize()
    return float(d_dt.item())


def test_noalloc_time_step_matches_context_entry_point():
    from hyperflow_gb300 import CartSolver, cases, lib
    L = lib()
    big = CartSolver(cases.quadrant_case(300, scheme="MUSCLHancock", limiter="MinBee"))
    small = CartSolver(cases.quadrant_case(70, ny=50, scheme="MUSCLHancock", limiter="VanLeer"))
    for s, n, ny, steps in ((big, 300, 300, 4), (small, 70, 50, 13)):
        s.run(steps)
        s.apply_bcs()
        U = s.state(0)                       # ghosts filled, as TimeStep sees them
        calls = s.time()[1]
        dt_ref = s.calculate_time_step()     # the existing entry point, call number `calls`
        ty, tx = U.shape[1:]
        got = _noalloc_dt(L, _device_copy(U), tx, ty, 1.0 / n, 1.0 / ny, calls)
        assert got == dt_ref, (got, dt_ref)


def test_noalloc_two_calls_in_a_row_and_limits():
    from hyperflow_gb300 import CartSolver, cases, lib
    L = lib()
    s = CartSolver(cases.quadrant_case(128, scheme="MUSCLHancock", limiter="MinBee"))
    got = []
    for _ in range(2):
        s.run(3)
        s.apply_bcs()
        U = s.state(0)
        calls = s.time()[1]
        ref = s.calculate_time_step()
        d = _device_copy(U)
        got.append((_noalloc_dt(L, d, U.shape[2], U.shape[1], 1 / 128, 1 / 128, calls), ref))
    for g, r in got:
        assert g == r
    import torch
    d_dt = torch.zeros(1, dtype=torch.float64, device="cuda")
    too_big = 4100
    st = L.hf_time_step_noalloc(d.data_ptr(), too_big, too_big, too_big, 1.0, 1.0, 1.4, 0.8, 0,
                                d_dt.data_ptr(), None)
    assert st == 8   # HF_ERR_TOO_LARGE, rejected before any launch
