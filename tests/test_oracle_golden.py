"""The oracle (C restatement, oracle/hf_oracle.c) against the golden fixtures the
reference itself produced (tests/golden/make_golden.py): bit-exact, every state value,
every dt of the step stream and every TimeStep call."""
import math

import numpy as np
import pytest

from conftest import golden_cart_names, load_golden, GOLDEN


@pytest.mark.parametrize("name", golden_cart_names())
def test_oracle_matches_reference_fixture(name, port_lib):
    from oracle.oracle import Oracle
    g = load_golden(name)
    o = Oracle(g["case"], nthreads=4)
    dts = o.run(int(g["steps"]), clamp_t_end=bool(g["clamp"]))
    assert len(dts) == int(g["steps"])
    np.testing.assert_array_equal(dts, g["step_dts"])
    assert o.calls == len(g["calls"])
    assert o.t == float(g["t"])
    if "U0" in g:
        for b in range(int(g["nblocks"])):
            np.testing.assert_array_equal(o.state(b), g[f"U{b}"])
    else:
        U = o.state(0)
        idx = g["sample_idx"]
        np.testing.assert_array_equal(U[:, idx[0], idx[1]], g["sample"])
        assert [math.fsum(U[v].ravel()) for v in range(4)] == list(g["sums"])
        assert [math.fsum((U[v] * U[v]).ravel()) for v in range(4)] == list(g["sumsq"])


def test_oracle_hllc_fallback_branch_is_exercised(port_lib):
    """The vacuum fixtures drive the reference's HLLC "should not get here" zero-flux
    branch; the oracle must take it too (its state already matches bit for bit)."""
    from oracle.oracle import Oracle
    g = load_golden("mh_minbee_vacuum_hllc_fallback")
    o = Oracle(g["case"], nthreads=4)
    o.run(int(g["steps"]))
    assert o.hllc_errors > 0


def test_oracle_units_match_reference(port_lib):
    import ctypes as C
    d = np.load(f"{GOLDEN}/unit_hllc_limiter.npz")
    UL, UR, F, r, lim = d["UL"], d["UR"], d["F"], d["r"], d["lim"]
    for k in range(len(r)):
        for kind in range(2):
            a = port_lib.hfo_limiter(kind, float(r[k]))
            b = lim[kind, k]
            assert (a == b) or (np.isnan(a) and np.isnan(b)), (kind, r[k], a, b)
    out = np.zeros(4)
    for dirn in range(2):
        for k in range(len(UL)):
            a = np.ascontiguousarray(UL[k]); b = np.ascontiguousarray(UR[k])
            port_lib.hfo_hllc(1.4, a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), dirn,
                              out.ctypes.data_as(C.c_void_p))
            np.testing.assert_array_equal(out, F[dirn, k])
