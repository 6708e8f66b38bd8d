"""The bounds-checked build (-DHF_CHECKS; it stands in for compute-sanitizer's memory checks):
every global index that depends on a block's geometry or on mesh data -- ghost fill sources and
destinations, ghost and interior CFL reads, stencil and host-buffer stores, unstructured pair,
neighbour and edge indices -- is range-checked, and a violation sets the context's error word
(HF_DEV_BOUNDS) instead of touching memory.  Small cases of every path run in that build must
raise nothing and give exactly the normal build's results (the oracle's)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import sys, numpy as np
sys.path.insert(0, ROOT)
sys.path.insert(0, ROOT + "/tests")
import hyperflow_gb300 as H
from hyperflow_gb300 import CartSolver, UnsSolver, cases, meshgen, _lib
from oracle.oracle import Oracle
assert _lib.LIB_PATH.endswith("_checked.so"), _lib.LIB_PATH
import torch
for case in (cases.forward_facing_step_case(20, limiter="VanLeer"),
             cases.forward_facing_step_case(20, scheme="Godunov"),
             cases.quadrant_case(33, ny=11, scheme="MUSCLHancock", limiter="MinBee"),
             cases.quadrant_case(65, ny=21, scheme="Godunov")):
    s, o = CartSolver(case), Oracle(case)
    s.run(8, graph=True)
    s.apply_bcs(); s.advance(s.calculate_time_step())
    host = [torch.empty(s.state(b).shape, dtype=torch.float64).pin_memory().numpy() for b in range(s.nblocks)]
    for b in range(s.nblocks):
        host[b][...] = s.state(b)
    s.step_io(host)
    s.sync()
    o.run(10)
    for b in range(s.nblocks):
        np.testing.assert_array_equal(s.state(b), o.state(b))
        np.testing.assert_array_equal(host[b], o.state(b))
from conftest import GOLDEN
g = np.load(GOLDEN + "/uns_tri_hole_3k.npz", allow_pickle=True)
import json
for edge in (False, True):
    u = UnsSolver(json.loads(str(g["case"])), mesh_text=meshgen.hmsh_text(g["verts"], g["codes"]))
    u.set_edge_mode(edge)
    u.run(int(g["steps"]))
    if not edge:
        np.testing.assert_array_equal(u.state(), g["U"])
    u.sync()
print("checked build clean")
'''


@pytest.mark.gpu
def test_checked_build_raises_nothing_and_matches():
    from hyperflow_gb300 import _build
    _build.build(variant="checked")
    env = dict(os.environ, HF_LIB_VARIANT="checked")
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + CHILD], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0 and "checked build clean" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]
