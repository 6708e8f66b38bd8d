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


def _noalloc_dt(L, d_state, tx, ty, dx, dy, call_index, cfl=0.8, pitch=None):
    import torch
    d_dt = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = L.hf_time_step_noalloc(d_state.data_ptr(), tx, ty, pitch or tx, dx, dy, 1.4, cfl, call_index,
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


def _pitched(U, pad):
    """U ([4][ty][tx]) on the device in rows of tx + pad doubles; the padding holds a state far
    faster than any cell (density 1e-6, momentum 1e6), which would shrink dt if it were read"""
    import torch
    _, ty, tx = U.shape
    P = np.empty((4, ty, tx + pad))
    P[0, :, tx:], P[1, :, tx:], P[2, :, tx:], P[3, :, tx:] = 1e-6, 1e6, 1e6, 1e12
    P[:, :, :tx] = U
    return torch.from_numpy(P).cuda(), tx + pad


def test_noalloc_pitched_rows_skip_the_padding():
    """A block stored with rows longer than the block (pitch > total_x): only the block's
    cells are read, and dt equals the context entry point's, on two calls in a row."""
    from hyperflow_gb300 import CartSolver, cases, lib
    L = lib()
    s = CartSolver(cases.quadrant_case(90, ny=61, scheme="MUSCLHancock", limiter="VanLeer"))
    for pad in (1, 38):
        s.run(2)
        s.apply_bcs()
        U = s.state(0)
        calls = s.time()[1]
        ref = s.calculate_time_step()
        d, pitch = _pitched(U, pad)
        got = _noalloc_dt(L, d, U.shape[2], U.shape[1], 1 / 90, 1 / 61, calls, pitch=pitch)
        assert got == ref, (pad, got, ref)


def test_noalloc_at_the_cell_limit():
    """A block of exactly 16,777,216 cells (4092 x 4092 interior cells and 2 ghost layers: 4096
    CTAs, the most the scratch array holds) gives the context entry point's dt; one cell more is
    refused before any launch."""
    import torch
    from hyperflow_gb300 import CartSolver, cases, lib
    L = lib()
    n = 4092
    s = CartSolver(cases.quadrant_case(n, scheme="MUSCLHancock", limiter="MinBee"))
    s.run(1)
    s.apply_bcs()
    U = s.state(0)
    assert U.shape[1] * U.shape[2] == 16_777_216
    calls = s.time()[1]
    ref = s.calculate_time_step()
    d = _device_copy(U)
    del U
    got = _noalloc_dt(L, d, 4096, 4096, 1 / n, 1 / n, calls)
    assert got == ref, (got, ref)
    d_dt = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = L.hf_time_step_noalloc(d.data_ptr(), 16_777_217, 1, 16_777_217, 1.0, 1.0, 1.4, 0.8, 0,
                                d_dt.data_ptr(), None)
    assert st == 8   # HF_ERR_TOO_LARGE
