"""Batched MUSCL-Hancock (one persistent cooperative launch per run of steps): every case
must equal the reference step run on that case alone -- here the oracle, bit for bit --
for every launch configuration, with and without the CUDA graph."""
import numpy as np
import pytest


def test_manifest_matches_the_workload_spec():
    from hyperflow_gb300 import cases
    m = cases.batch_manifest(512, seed=0)
    assert len(m["cases"]) == 512
    sides = np.array([c["mesh"]["blocks"][0]["x_cells"] for c in m["cases"]])
    assert sides.min() >= 64 and sides.max() <= 1024
    # log-uniform: the median side is near sqrt(64 * 1024) = 256
    assert 200 < np.median(sides) < 330
    for c in m["cases"][:50]:
        ic = c["initial_condition"]
        assert 0.3 <= ic["x_interface"] <= 0.7 and 0.3 <= ic["y_interface"] <= 0.7
        for k in ("init_ne_state", "init_nw_state", "init_sw_state", "init_se_state"):
            r, u, v, p = ic[k]
            assert 0.1 <= r <= 2 and -1 <= u <= 1 and -1 <= v <= 1 and 0.1 <= p <= 10
        assert all(b["type"] == "Transmissive" for b in c["mesh"]["blocks"][0]["boundaries"].values())
    assert cases.batch_manifest(8, seed=3) == cases.batch_manifest(8, seed=3)


def _oracle_interior(case, steps):
    from oracle.oracle import Oracle
    o = Oracle(case, nthreads=4)
    o.run(steps)
    return o.state(0)[:, 2:-2, 2:-2], o.t


@pytest.mark.gpu
def test_batch_every_config_matches_oracle(port_lib):
    from hyperflow_gb300 import BatchSolver, cases
    from hyperflow_gb300.batch import configs
    m = cases.batch_manifest(10, seed=7, side_min=64, side_max=100)
    steps = 25
    ref = [_oracle_interior(c, steps) for c in m["cases"]]
    for k in range(len(configs())):
        b = BatchSolver(m)
        b.set_config(k)
        b.run(steps, graph=False)
        b.sync()
        for i in range(b.ninstances):
            np.testing.assert_array_equal(b.state(i), ref[i][0], err_msg=f"config {k} case {i}")
            assert b.instance_time(i)[0] == ref[i][1]
        assert b.counters()["calls"] == 2 * steps


@pytest.mark.gpu
def test_batch_graph_and_chunks_equal_single_launch(port_lib):
    from hyperflow_gb300 import BatchSolver, cases
    m = cases.batch_manifest(6, seed=11, side_min=64, side_max=90, limiter="VanLeer")
    a, b = BatchSolver(m), BatchSolver(m)
    a.run(30, graph=False)
    for _ in range(3):
        b.run(10, graph=True)       # one captured 10-step launch, replayed
    b.sync()
    for i in range(a.ninstances):
        np.testing.assert_array_equal(a.state(i), b.state(i))
    ref, _ = _oracle_interior(m["cases"][0], 30)
    np.testing.assert_array_equal(a.state(0), ref)


@pytest.mark.gpu
def test_batch_autotune_restores_state(port_lib):
    from hyperflow_gb300 import BatchSolver, cases
    m = cases.batch_manifest(8, seed=2, side_min=64, side_max=128)
    b = BatchSolver(m)
    b.run(3, graph=False)
    before = [b.state(i) for i in range(b.ninstances)]
    best, ms = b.autotune(steps_per_trial=2)
    assert 0 <= best < len(ms) and (ms > 0).all()
    for i in range(b.ninstances):
        np.testing.assert_array_equal(b.state(i), before[i])
    b.run(5, graph=True)
    b.sync()
    ref, _ = _oracle_interior(m["cases"][1], 8)
    np.testing.assert_array_equal(b.state(1), ref)


@pytest.mark.gpu
def test_batch_full_workload_sample_matches_oracle(port_lib):
    """The 512-case workload (sides 64..1024) to its 500 steps in one graph-captured persistent
    launch; 16 seeded cases plus the smallest and the largest (side 1010) checked against the
    oracle run on each case alone, bit for bit, with each case's own time."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    from hyperflow_gb300 import BatchSolver, cases
    from oracle.oracle import Oracle
    steps = 500
    m = cases.batch_manifest(512, seed=0)
    b = BatchSolver(m)
    assert b.ninstances == 512
    b.run(steps, graph=True)
    b.sync()
    sides = np.array(b.sides)
    assert sides.max() == 1010 and sides.min() == 64     # this seed's extremes (the range is 64..1024)
    rng = np.random.default_rng(1)
    pick = sorted(set(rng.choice(512, 16, replace=False).tolist()) | {int(sides.argmin()), int(sides.argmax())})
    threads = max(1, (os.cpu_count() or 4) // 4)

    def oracle_run(i):
        o = Oracle(m["cases"][i], nthreads=threads)
        o.run(steps)
        return i, o.state(0)[:, 2:-2, 2:-2], o.t

    with ThreadPoolExecutor(max_workers=4) as ex:
        for i, ref, t in ex.map(oracle_run, pick):
            np.testing.assert_array_equal(b.state(i), ref, err_msg=f"case {i} side {sides[i]}")
            assert b.instance_time(i)[0] == t


@pytest.mark.gpu
def test_batch_godunov_every_config_matches_oracle(port_lib):
    """Batched Godunov cases (one TimeStep call per step) equal the oracle, bit for bit."""
    from hyperflow_gb300 import BatchSolver, cases
    from hyperflow_gb300.batch import configs
    m = cases.batch_manifest(7, seed=5, side_min=40, side_max=100, scheme="Godunov")
    steps = 30
    ref = []
    for c in m["cases"]:
        from oracle.oracle import Oracle
        o = Oracle(c, nthreads=4)
        o.run(steps)
        ref.append((o.state(0)[:, 1:-1, 1:-1], o.t))
    for k in range(len(configs())):
        b = BatchSolver(m)
        b.set_config(k)
        b.run(steps, graph=k % 2 == 0)
        b.sync()
        for i in range(b.ninstances):
            np.testing.assert_array_equal(b.state(i), ref[i][0], err_msg=f"config {k} case {i}")
            assert b.instance_time(i)[0] == ref[i][1]
        assert b.counters()["calls"] == steps


@pytest.mark.gpu
def test_batch_of_one_runs_the_256_godunov_workload(port_lib):
    """The 256^2 Godunov quadrant problem x 200 steps as a batch of one (the whole run in one
    persistent launch) equals the per-block solver and the oracle's dt stream end state."""
    from hyperflow_gb300 import BatchSolver, CartSolver, cases
    case = cases.quadrant_case(256)
    b = BatchSolver({"cases": [case]})
    b.run(200, graph=True)
    b.sync()
    s = CartSolver(case)
    s.run(200)
    np.testing.assert_array_equal(b.state(0), s.state(0)[:, 1:-1, 1:-1])
    assert b.instance_time(0)[0] == s.time()[0]


@pytest.mark.gpu
def test_batch_records_the_earliest_nonpositive_cell(port_lib):
    """Eight small Riemann problems at CFL 0.8 (unstable for 2D flow): cases 7 and 2 leave a cell
    with non-positive pressure at steps 29 and 31.  The batch records the least (step, case, j, i),
    equal to the oracle's per-case records, runs on as the reference does (every state equals the
    oracle's, NaNs included), and clearing forgets the record."""
    from oracle.oracle import Oracle
    from hyperflow_gb300 import BatchSolver, cases
    m = cases.batch_manifest(8, seed=4, side_min=48, side_max=80, cfl=0.8)
    steps = 40
    recs, ref = [], []
    for k, c in enumerate(m["cases"]):
        o = Oracle(c, nthreads=4)
        o.run(steps)
        ref.append(o.state(0)[:, 2:-2, 2:-2])
        if o.first_nonpos is not None:
            r = o.first_nonpos
            recs.append((r["step"], k, r["j"], r["i"]))
    assert [(s, k) for s, k, _, _ in sorted(recs)] == [(29, 7), (31, 2)]
    b = BatchSolver(m)
    b.run(28)
    assert b.last_nonpositive_cell() is None
    b.run(steps - 28)
    s, k, j, i = min(recs)
    assert b.last_nonpositive_cell() == {"step": s, "case": k, "j": j, "i": i}
    for n in range(b.ninstances):
        np.testing.assert_array_equal(b.state(n), ref[n], err_msg=f"case {n}")
    b.clear_error_cell()
    assert b.last_nonpositive_cell() is None
