"""GPU frame output and checkpoint/restart through the C ABI.

Frames: the device loop with Simulation::solve's frame dt clamp and output cadence writes,
bit for bit, the frames the oracle's solve takes, and their CSV text hashes to what the
reference's own solve wrote; a ring of two slots (the loop pausing for the host) gives the
same frames.  Checkpoints: a run restored from a checkpoint continues bit for bit."""
import hashlib
import os

import numpy as np
import pytest

from test_frames import frame_fixtures, load_frames

pytestmark = pytest.mark.gpu


def _solve_frames(case, tmp_path, ring_slots, fmt="hfb"):
    from hyperflow_gb300 import CartSolver, frames as fr
    s = CartSolver(case)
    steps = s.solve(out_dir=str(tmp_path), fmt=fmt, ring_slots=ring_slots)
    paths = sorted(s.frame_paths)
    return s, steps, paths


@pytest.mark.parametrize("name", frame_fixtures())
def test_gpu_frames_equal_oracle_and_reference(name, tmp_path, port_lib):
    from hyperflow_gb300 import frames as fr
    from oracle.oracle import Oracle
    g = load_frames(name)
    o = Oracle(g["case"])
    _, labels, oframes = o.solve(max_frames=len(g["csv_sha256"]) + 1)
    s, steps, paths = _solve_frames(g["case"], tmp_path, ring_slots=8)
    assert len(paths) == len(g["csv_sha256"]) == len(oframes)
    t, calls, _ = s.time()
    assert calls == len(g["calls"])
    for b in range(int(g["nblocks"])):
        np.testing.assert_array_equal(s.state(b), g[f"U{b}"])
    every = 1 if len(paths) < 100 else 37
    for k, p in enumerate(paths):
        head, blocks = fr.read_frame(p)
        assert head["index"] == k and head["t"] == labels[k], k
        for a, b in zip(blocks, oframes[k]):
            np.testing.assert_array_equal(a, b)
        if k % every == 0 or k == len(paths) - 1:
            h = hashlib.sha256(fr.csv_text(head, blocks).encode()).hexdigest()
            assert h == g["csv_sha256"][k], k


def test_gpu_frames_with_a_two_slot_ring(tmp_path):
    """600 frames through a ring of two: the loop pauses for every frame and resumes."""
    from hyperflow_gb300 import frames as fr
    g = load_frames("sphericalrp_godunov_hllc_50x50")
    _, _, p8 = _solve_frames(g["case"], tmp_path / "r8", ring_slots=8)
    s2, _, p2 = _solve_frames(g["case"], tmp_path / "r2", ring_slots=2)
    assert len(p8) == len(p2) == len(g["csv_sha256"])
    for a, b in zip(p8, p2):
        ha, ba = fr.read_frame(a)
        hb, bb = fr.read_frame(b)
        assert ha["t"] == hb["t"]
        np.testing.assert_array_equal(ba[0], bb[0])
    np.testing.assert_array_equal(s2.state(0), g["U0"])


def test_gpu_csv_frames_are_the_reference_text(tmp_path):
    g = load_frames("toro_shock_tube_01_muscl_hancock_vanleer_hllc_100x5")
    _, _, paths = _solve_frames(g["case"], tmp_path, ring_slots=4, fmt="csv")
    assert [hashlib.sha256(open(p, "rb").read()).hexdigest() for p in paths] == list(g["csv_sha256"])


@pytest.mark.parametrize("scheme", ["Godunov", "MUSCLHancock"])
def test_gpu_checkpoint_restart_is_bit_exact(scheme, tmp_path):
    from hyperflow_gb300 import CartSolver, cases
    case = cases.forward_facing_step_case(40, scheme=scheme) if scheme == "Godunov" else \
        cases.forward_facing_step_case(40, limiter="VanLeer")
    a = CartSolver(case)
    a.run(7)                       # inside the 0.2 * cfl start-up calls
    path = str(tmp_path / "ck.bin")
    a.save_checkpoint(path)
    a.run(30)
    b = CartSolver(case)
    b.load_checkpoint(path)
    b.run(30)
    assert a.time() == b.time()
    for k in range(a.nblocks):
        np.testing.assert_array_equal(a.state(k), b.state(k))
    # per-step API after a restore as well
    b.load_checkpoint(path)
    c_dts = [b.step() for _ in range(5)]
    a.load_checkpoint(path)
    assert [a.step() for _ in range(5)] == c_dts


def test_gpu_checkpoint_rejects_another_case(tmp_path):
    from hyperflow_gb300 import CartSolver, HyperFlowError, cases
    a = CartSolver(cases.quadrant_case(32))
    blob = a.checkpoint()
    b = CartSolver(cases.quadrant_case(40))
    with pytest.raises(HyperFlowError):
        b.restore(blob)
    with pytest.raises(HyperFlowError):
        a.restore(blob[:100])


def _run_popping(s, n, out):
    """n device-loop steps, popping frames whenever the ring pauses the loop"""
    done = 0
    while done < n:
        k = s.run(n - done, clamp_t_end=True)
        done += k
        popped = 0
        while s.frames_pending():
            out.append(s.pop_frame())
            popped += 1
        if k == 0 and popped == 0:
            break
    return done


def test_gpu_checkpoint_carries_the_frame_cadence(tmp_path):
    """Frames taken by a run split by a checkpoint equal those of the unbroken run."""
    from hyperflow_gb300 import CartSolver
    g = load_frames("toro_shock_tube_01_godunov_hllc_100x5")
    full = CartSolver(g["case"])
    full.enable_frames(4)
    want = []
    assert _run_popping(full, 60, want) == 60
    a = CartSolver(g["case"])
    a.enable_frames(4)
    got = []
    assert _run_popping(a, 25, got) == 25
    blob = a.checkpoint()
    b = CartSolver(g["case"])
    b.enable_frames(4)
    b.restore(blob)
    assert _run_popping(b, 35, got) == 35
    assert len(want) > 5
    assert [(i, t) for i, t, _ in got] == [(i, t) for i, t, _ in want]
    for (_, _, x), (_, _, y) in zip(got, want):
        np.testing.assert_array_equal(x[0], y[0])
    np.testing.assert_array_equal(b.state(0), full.state(0))


@pytest.mark.parametrize("name", ["quad_channel_240", "tri_hole_3k"])
@pytest.mark.parametrize("ring", [8, 2])
def test_gpu_uns_frames_equal_oracle_and_reference(name, ring, tmp_path, port_lib):
    from hyperflow_gb300 import UnsSolver, frames as fr, meshgen
    from test_frames import load_uns_frames, uns_oracle_solve
    g = load_uns_frames(name)
    U, labels, oframes = uns_oracle_solve(g)
    s = UnsSolver(g["case"], mesh_text=meshgen.hmsh_text(g["verts"], g["codes"]))
    np.testing.assert_array_equal(s.centroids(), g["centroids"])
    s.solve(out_dir=str(tmp_path), ring_slots=ring)
    np.testing.assert_array_equal(s.state(), g["U"])
    paths = sorted(s.frame_paths)
    assert len(paths) == len(g["csv_sha256"]) == len(oframes)
    cen = s.centroids()
    for k, p in enumerate(paths):
        head, (Uk,) = fr.read_frame(p)
        assert head["index"] == k and head["t"] == labels[k]
        np.testing.assert_array_equal(Uk, oframes[k])
        h = hashlib.sha256(fr.uns_csv_text(head, Uk, cen).encode()).hexdigest()
        assert h == g["csv_sha256"][k], k


@pytest.mark.parametrize("scheme", ["MUSCLHancock", "Godunov"])
def test_gpu_multiblock_frames_equal_oracle(scheme, tmp_path, port_lib):
    """Frames of the 3-block forward-facing step (internal, inflow, reflective and
    transmissive sides) against the oracle's Simulation::solve, bit for bit."""
    from hyperflow_gb300 import CartSolver, cases, frames as fr
    from oracle.oracle import Oracle
    case = cases.forward_facing_step_case(30, scheme=scheme, t_end=0.05)
    case["simulation"]["animation"] = {"duration": 1.0, "fps": 16.0}
    o = Oracle(case, nthreads=4)
    _, labels, oframes = o.solve(max_frames=64)
    s = CartSolver(case)
    s.solve(out_dir=str(tmp_path), ring_slots=4)
    paths = sorted(s.frame_paths)
    assert len(paths) == len(oframes) > 10
    for k, p in enumerate(paths):
        head, blocks = fr.read_frame(p)
        assert head["index"] == k and head["t"] == labels[k]
        for a, b in zip(blocks, oframes[k]):
            np.testing.assert_array_equal(a, b)
    for b in range(s.nblocks):
        np.testing.assert_array_equal(s.state(b), o.state(b))


_CRASHER = r'''
import os, sys
sys.path.insert(0, ROOT)
from hyperflow_gb300 import CartSolver, cases
s = CartSolver(cases.forward_facing_step_case(20, limiter="VanLeer"))
for k in range(1, 100):
    s.run(5)
    blob = s.checkpoint()                  # synchronises: no kernel is in flight after this
    tmp = PATH + ".tmp"
    with open(tmp, "wb") as f:
        f.write(blob)
    os.replace(tmp, PATH)                  # the checkpoint file is always a whole one
    if k == 3:
        os._exit(17)                       # the "rank" dies here, between steps, without cleanup
'''


def test_gpu_resume_after_a_process_dies_between_steps(tmp_path):
    """A process that checkpoints every 5 steps dies abruptly (between steps, after its third
    checkpoint, no cleanup); a new solver restored from the last checkpoint file and run on
    equals an uninterrupted run bit for bit."""
    import subprocess
    import sys
    from hyperflow_gb300 import CartSolver, cases
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = str(tmp_path / "ck.bin")
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\nPATH = %r\n" % (root, path) + _CRASHER],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 17, r.stderr[-2000:]
    case = cases.forward_facing_step_case(20, limiter="VanLeer")
    b = CartSolver(case)
    b.load_checkpoint(path)
    b.run(25)
    a = CartSolver(case)
    a.run(40)
    assert a.time() == b.time()
    for k in range(a.nblocks):
        np.testing.assert_array_equal(a.state(k), b.state(k))
