"""Where the reference tree is present (oracle/_ref built from it), the oracle is also
compared live against the reference on cases not stored as fixtures."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="reference build (oracle/_ref) absent")


@pytest.mark.parametrize("n,ny,scheme,lim,bc,steps", [
    (24, 31, "Godunov", None, "Transmissive", 30),
    (26, 20, "MUSCLHancock", "MinBee", "Reflective", 30),
    (20, 26, "MUSCLHancock", "VanLeer", "Transmissive", 30),
])
def test_live_quadrant(n, ny, scheme, lim, bc, steps, port_lib):
    from hyperflow_gb300 import cases
    case = cases.quadrant_case(n, ny=ny, scheme=scheme, limiter=lim, bc=bc, split=(0.37, 0.58))
    ref = oracle.RefCart(case)
    ref.run(steps)
    o = oracle.Oracle(case)
    dts = o.run(steps)
    np.testing.assert_array_equal(dts, ref.step_dts())
    np.testing.assert_array_equal(o.state(0), ref.state(0))


def test_live_ffs_multiblock(port_lib):
    from hyperflow_gb300 import cases
    case = cases.forward_facing_step_case(25, limiter="VanLeer")
    ref = oracle.RefCart(case)
    ref.run(25)
    o = oracle.Oracle(case)
    o.run(25)
    for b in range(3):
        np.testing.assert_array_equal(o.state(b), ref.state(b))
    assert o.calls == len(ref.calls())
