"""Unstructured Godunov + HLLC step (src/fvm_2d_uns): oracle against the reference's
fixtures (CPU), and the CUDA path against both (GPU), bit for bit."""
import glob
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def uns_names():
    return sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "uns_*.npz")))


def load(name):
    d = np.load(os.path.join(GOLDEN, f"uns_{name}.npz"))
    g = {k: d[k] for k in d.files}
    g["case"] = json.loads(str(g["case"]))
    return g


def _inlet(case):
    from oracle.oracle import prim_to_cons
    return prim_to_cons(case["mesh"]["boundaries"]["inlet"])


@pytest.mark.parametrize("name", uns_names())
def test_uns_oracle_matches_reference_fixture(name, port_lib):
    from oracle import oracle
    from hyperflow_gb300 import meshgen
    g = load(name)
    V, codes = g["verts"], g["codes"]
    nbr = oracle.ref_neighbours(V, codes)[0]
    np.testing.assert_array_equal(nbr, g["nbr"])
    nverts = np.full(len(V), V.shape[1], np.int32)
    ang, ln, area, rin = oracle.uns_geometry(nverts, V.reshape(-1, 2))
    for a, b in ((ang, "angle"), (ln, "length"), (area, "area"), (rin, "rin")):
        np.testing.assert_array_equal(a, g[b])
    U = np.zeros((4, len(V)))
    U[:] = oracle.prim_to_cons(g["case"]["initial_condition"]["init_state"])[:, None]
    ps = np.concatenate([[0], np.cumsum(nverts)]).astype(np.int32)
    dts, calls = oracle.uns_run(1.4, g["case"]["simulation"]["cfl"], 0, ps, nbr, ang, ln, area, rin,
                                _inlet(g["case"]), U, int(g["steps"]), nthreads=4)
    np.testing.assert_array_equal(dts, g["dts"])
    np.testing.assert_array_equal(U, g["U"])


def test_mesh_text_round_trip():
    from hyperflow_gb300 import meshgen
    V, codes = meshgen.jittered_hole_mesh(500, seed=9)
    text = meshgen.hmsh_text(V, codes)
    lines = text.splitlines()
    assert lines[0] == "CELLS" and int(lines[1]) == len(V)
    back = np.array([[float(x) for x in l.split()] for l in lines[2:2 + len(V)]]).reshape(V.shape)
    np.testing.assert_array_equal(back, V)


def test_mesh_binary_round_trip():
    """The binary mesh format holds exactly the text format's content."""
    from hyperflow_gb300 import meshgen
    V, codes = meshgen.jittered_hole_mesh(500, seed=9)
    data = meshgen.hmshb_bytes(V, codes)
    assert data[:8] == b"HFMESHB1" and len(data) % 8 == 0
    v2, c2 = meshgen.read_hmshb(data)
    np.testing.assert_array_equal(np.array(v2), V)
    np.testing.assert_array_equal(np.array(c2), codes)
    v3, c3 = meshgen.read_hmsh(meshgen.hmsh_text(V, codes))
    assert v3 == v2 and c3 == c2
    with pytest.raises(ValueError):
        meshgen.read_hmshb(data[:-8])


def test_generator_is_canonical():
    from hyperflow_gb300 import meshgen
    a = meshgen.jittered_hole_mesh(2000, seed=5)
    b = meshgen.jittered_hole_mesh(2000, seed=5)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    V = a[0]
    cross = (V[:, 1, 0] - V[:, 0, 0]) * (V[:, 2, 1] - V[:, 0, 1]) - \
            (V[:, 1, 1] - V[:, 0, 1]) * (V[:, 2, 0] - V[:, 0, 0])
    assert (cross > 0).all()                       # counter-clockwise
    assert set(np.unique(a[1])) == {0, -1, -2, -3}  # interior, wall, outflow, inlet


@pytest.mark.gpu
@pytest.mark.parametrize("name", uns_names())
def test_uns_gpu_matches_reference_fixture(name):
    from hyperflow_gb300 import UnsSolver, meshgen
    g = load(name)
    s = UnsSolver(g["case"], mesh_text=meshgen.hmsh_text(g["verts"], g["codes"]))
    m = s.mesh_arrays()
    np.testing.assert_array_equal(m["nbr"], g["nbr"])
    for k in ("angle", "length", "area", "rin"):
        np.testing.assert_array_equal(m[k], g[k])
    dts = []
    for _ in range(int(g["steps"])):
        dts.append(s.calculate_time_step())
        s.advance(dts[-1])
    np.testing.assert_array_equal(np.array(dts), g["dts"])
    np.testing.assert_array_equal(s.state(), g["U"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", uns_names())
def test_uns_gpu_binary_mesh_equals_text(name, tmp_path):
    """The same mesh in the binary format, in memory and as mesh.file, loads to the same pairs,
    neighbours, geometry and centroids and steps to the same states; malformed binary meshes
    are refused before any device work."""
    from hyperflow_gb300 import HyperFlowError, UnsSolver, meshgen
    g = load(name)
    text = meshgen.hmsh_text(g["verts"], g["codes"])
    data = meshgen.hmshb_bytes(g["verts"], g["codes"])
    path = tmp_path / "mesh.hmshb"
    path.write_bytes(data)
    case = json.loads(json.dumps(g["case"]))
    case["mesh"]["file"] = str(path)
    a, b, c = UnsSolver(g["case"], mesh_text=text), UnsSolver(g["case"], mesh_text=data), UnsSolver(case)
    ma = a.mesh_arrays()
    for s in (b, c):
        m = s.mesh_arrays()
        for k in ma:
            np.testing.assert_array_equal(m[k], ma[k], err_msg=k)
        np.testing.assert_array_equal(s.centroids(), a.centroids())
    for s in (a, b, c):
        s.run(int(g["steps"]))
    np.testing.assert_array_equal(b.state(), g["U"])
    np.testing.assert_array_equal(c.state(), g["U"])
    bad_count = data[:24] + np.array([5], "<i4").tobytes() + data[28:]   # first cell: 5 vertices
    for broken in (data[:-8], data[:20], bad_count):
        with pytest.raises(HyperFlowError):
            UnsSolver(g["case"], mesh_text=broken)


@pytest.mark.gpu
def test_uns_gpu_device_loop_equals_piecewise():
    from hyperflow_gb300 import UnsSolver, meshgen
    g = load("tri_hole_3k")
    text = meshgen.hmsh_text(g["verts"], g["codes"])
    a, b = UnsSolver(g["case"], mesh_text=text), UnsSolver(g["case"], mesh_text=text)
    a.run(int(g["steps"]), graph=True)
    np.testing.assert_array_equal(a.state(), g["U"])
    b.run(int(g["steps"]), graph=False)
    np.testing.assert_array_equal(b.state(), g["U"])
    assert a.time()[1] == int(g["steps"])


@pytest.mark.gpu
def test_uns_gpu_full_size_matches_oracle(tmp_path):
    """The ~1M-triangle circular-hole channel (Mach 2, CFL 0.5), read from a mesh file as the
    reference reads it, to the configured 2000 steps against the oracle on all host cores: the
    per-pair mode bit for bit, and the edge-based mode (the benchmarked one; its partner-side
    flux is the owner's negated) within 1e-10 relative in every variable."""
    from hyperflow_gb300 import UnsSolver, meshgen
    from oracle import oracle
    V, codes = meshgen.jittered_hole_mesh(1_000_000, seed=0)
    path = tmp_path / "channel.hmsh"
    meshgen.write_hmsh(str(path), V, codes)
    case = meshgen.channel_case(str(path), cfl=0.5)
    s = UnsSolver(case)
    assert 950_000 < s.ncells < 1_050_000
    assert s.unmatched_pairs() == (0, -1)
    m = s.mesh_arrays()
    steps = 2000
    s.run(steps)
    e = UnsSolver(case)
    e.set_edge_mode(True)
    e.run(steps)
    U = np.zeros((4, s.ncells))
    U[:] = oracle.prim_to_cons(case["initial_condition"]["init_state"])[:, None]
    dts, _ = oracle.uns_run(1.4, 0.5, 0, m["pair_start"], m["nbr"], m["angle"], m["length"], m["area"],
                            m["rin"], _inlet(case), U, steps, nthreads=os.cpu_count() or 4)
    t = 0.0
    for dt in dts:
        t += float(dt)
    assert s.time()[0] == t and e.time()[0] != 0.0
    np.testing.assert_array_equal(s.state(), U)
    rel = np.abs(e.state() - U) / np.abs(U).max(axis=1, keepdims=True)
    assert rel.max() <= 1e-10, rel.max()


@pytest.mark.gpu
def test_uns_edge_mode_within_tolerance(port_lib):
    """Edge-based mode (one HLLC per unique interior edge) against the per-side oracle after
    2000 steps: the lower-indexed cell's flux is the reference's own; the other cell's is the
    negation, which differs by rounding -- within 1e-10 relative."""
    from hyperflow_gb300 import UnsSolver, meshgen
    from oracle import oracle
    g = load("tri_hole_3k")
    s = UnsSolver(g["case"], mesh_text=meshgen.hmsh_text(g["verts"], g["codes"]))
    s.set_edge_mode(True)
    steps = 2000
    s.run(steps)
    m = s.mesh_arrays()
    U = np.zeros((4, s.ncells))
    U[:] = oracle.prim_to_cons(g["case"]["initial_condition"]["init_state"])[:, None]
    oracle.uns_run(1.4, g["case"]["simulation"]["cfl"], 0, m["pair_start"], m["nbr"], m["angle"],
                   m["length"], m["area"], m["rin"], _inlet(g["case"]), U, steps, nthreads=4)
    V = s.state()
    scale = np.abs(U).max(axis=1, keepdims=True)
    rel = np.abs(V - U) / scale
    assert rel.max() <= 1e-10, rel.max()
    s.set_edge_mode(False)   # the parity path is still available on the same solver


@pytest.mark.gpu
def test_uns_gpu_checkpoint_restart_is_bit_exact():
    """A run restored from a checkpoint taken inside the start-up calls continues bit for bit,
    through the device loop and the per-step API; another mesh's checkpoint is refused."""
    from hyperflow_gb300 import HyperFlowError, UnsSolver, meshgen
    g = load("tri_hole_3k")
    text = meshgen.hmsh_text(g["verts"], g["codes"])
    a = UnsSolver(g["case"], mesh_text=text)
    a.run(4)
    blob = a.checkpoint()
    a.run(40)
    b = UnsSolver(g["case"], mesh_text=text)
    b.restore(blob)
    b.run(40)
    assert a.time() == b.time()
    np.testing.assert_array_equal(a.state(), b.state())
    b.restore(blob)
    dts = []
    for _ in range(5):
        dt = b.calculate_time_step()
        b.advance(dt)
        dts.append(dt)
    a.restore(blob)
    for dt in dts:
        assert a.calculate_time_step() == dt
        a.advance(dt)
    np.testing.assert_array_equal(a.state(), b.state())
    other = UnsSolver(g["case"], mesh_text=meshgen.hmsh_text(*meshgen.jittered_hole_mesh(4000, seed=1)))
    with pytest.raises(HyperFlowError):
        other.restore(blob)
    with pytest.raises(HyperFlowError):
        a.restore(blob[:64])


@pytest.mark.gpu
def test_uns_gpu_negative_pressure_cell_and_strict_mode():
    """A cell with negative total energy: the NaNs spread exactly as in the oracle, the
    earliest zero-flux pair is at step 0 on that cell or a neighbour, and strict mode stops
    the device loop after that step."""
    from hyperflow_gb300 import HyperFlowError, UnsSolver, meshgen
    from oracle import oracle
    g = load("tri_hole_3k")
    text = meshgen.hmsh_text(g["verts"], g["codes"])
    s = UnsSolver(g["case"], mesh_text=text)
    U = s.state()
    U[3, 100] = -1.0
    s.set_state(U)
    s.run(3)
    m = s.mesh_arrays()
    V = U.copy()
    oracle.uns_run(1.4, g["case"]["simulation"]["cfl"], 0, m["pair_start"], m["nbr"], m["angle"],
                   m["length"], m["area"], m["rin"], _inlet(g["case"]), V, 3)
    np.testing.assert_array_equal(s.state(), V)
    assert s.hllc_errors() > 0
    bad = s.last_error_cell()
    nbrs = {100} | {int(k) for k in m["nbr"][m["pair_start"][100]:m["pair_start"][101]] if k >= 0}
    assert bad["step"] == 0 and bad["cell"] in nbrs
    # the earliest non-positive cell: the oracle's state after one step, scanned in cell order
    W = U.copy()
    oracle.uns_run(1.4, g["case"]["simulation"]["cfl"], 0, m["pair_start"], m["nbr"], m["angle"],
                   m["length"], m["area"], m["rin"], _inlet(g["case"]), W, 1)
    first = oracle.uns_first_nonpositive(1.4, W)
    assert first is not None
    assert s.last_nonpositive_cell() == {"step": 0, "cell": first}
    t = UnsSolver(g["case"], mesh_text=text)
    t.set_state(U)
    t.set_strict(True)
    with pytest.raises(HyperFlowError, match="zero flux"):
        t.run(5)
    assert t.time()[1] == 1
    s.clear_error_cell()
    assert s.last_error_cell() is None and s.last_nonpositive_cell() is None


@pytest.mark.gpu
def test_uns_gpu_adaptor_call_sequence_matches_oracle():
    """The unstructured adaptor's call sequence (hyperflow_gb300/adaptor/gpu_uns_scheme.h):
    per step the cells' values are uploaded, the device forms dt (TimeStep), advances, and the
    values are downloaded -- bit for bit against the oracle stepping its own copy."""
    from hyperflow_gb300 import UnsSolver, meshgen
    from oracle import oracle
    g = load("tri_hole_3k")
    s = UnsSolver(g["case"], mesh_text=meshgen.hmsh_text(g["verts"], g["codes"]))
    m = s.mesh_arrays()
    U = s.state().copy()
    host = U.copy()
    calls = 0
    for _ in range(15):
        dts, calls = oracle.uns_run(1.4, g["case"]["simulation"]["cfl"], calls, m["pair_start"], m["nbr"],
                                    m["angle"], m["length"], m["area"], m["rin"], _inlet(g["case"]), U, 1)
        s.set_state(host)                       # GpuUnsTimeStep: upload the cells' values
        dt = s.calculate_time_step()
        assert dt == float(dts[0])
        s.advance(dt)                           # GpuUnsForwardEuler
        host = s.state()
    np.testing.assert_array_equal(host, U)
