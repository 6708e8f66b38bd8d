"""The integer-pipe FP64 division and square root used by the kernels equal the hardware
IEEE operations,
bit for bit, on hundreds of millions of generated operand pairs per operand class."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4, 5, 6, 7])
def test_division_matches_hardware(mode):
    from hyperflow_gb300 import lib
    bad = C.c_int64()
    first = np.zeros(4)
    n = 400_000_000 if mode in (1, 2) else 100_000_000
    assert lib().hf_diag_div_check(12345 + mode, n, mode, C.byref(bad), first.ctypes.data) == 0
    assert bad.value == 0, f"mode {mode}: {bad.value} mismatches, first a,b,got,want = {first.tolist()}"
