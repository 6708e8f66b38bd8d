"""GPU parity of the Cartesian time step through the C ABI: bit-exact against the
reference's golden fixtures and against the oracle (the C restatement) on the same
inputs, at fixture sizes and at the full benchmark sizes."""
import math

import numpy as np
import pytest

from conftest import golden_cart_names, load_golden

pytestmark = pytest.mark.gpu


def _solver(case):
    from hyperflow_gb300 import CartSolver
    return CartSolver(case)


@pytest.mark.parametrize("name", golden_cart_names())
def test_gpu_matches_reference_fixture(name):
    g = load_golden(name)
    s = _solver(g["case"])
    taken = s.run(int(g["steps"]), clamp_t_end=bool(g["clamp"]))
    assert taken == int(g["steps"])
    t, calls, _ = s.time()
    assert t == float(g["t"])
    assert calls == len(g["calls"])
    if "U0" in g:
        for b in range(int(g["nblocks"])):
            np.testing.assert_array_equal(s.state(b), g[f"U{b}"])
    else:
        U = s.state(0)
        idx = g["sample_idx"]
        np.testing.assert_array_equal(U[:, idx[0], idx[1]], g["sample"])
        assert [math.fsum(U[v].ravel()) for v in range(4)] == list(g["sums"])
        assert [math.fsum((U[v] * U[v]).ravel()) for v in range(4)] == list(g["sumsq"])


@pytest.mark.parametrize("name", ["godunov_quad_48", "mh_minbee_quad_48", "ffs_vanleer_dx1_40",
                                  "mh_minbee_vacuum_hllc_fallback"])
def test_gpu_dt_stream_step_by_step(name, port_lib):
    """hf_step returns each step's dt: the whole stream equals the reference's."""
    g = load_golden(name)
    s = _solver(g["case"])
    dts = [s.step() for _ in range(int(g["steps"]))]
    np.testing.assert_array_equal(np.array(dts), g["step_dts"])


def test_gpu_hllc_fallback_count_matches_oracle(port_lib):
    from oracle.oracle import Oracle
    g = load_golden("mh_vanleer_vacuum_hllc_fallback")
    o = Oracle(g["case"], nthreads=4)
    o.run(int(g["steps"]))
    s = _solver(g["case"])
    s.run(int(g["steps"]))
    assert o.hllc_errors > 0
    assert s.hllc_errors() == o.hllc_errors


def test_gpu_first_zero_flux_face_matches_oracle(port_lib):
    """The earliest zero-flux face (step, block, direction, j, i) equals the oracle's on the
    vacuum-forming fixture; clearing forgets it."""
    from oracle.oracle import Oracle
    g = load_golden("mh_vanleer_vacuum_hllc_fallback")
    o = Oracle(g["case"], nthreads=4)
    o.run(int(g["steps"]))
    s = _solver(g["case"])
    s.run(int(g["steps"]))
    assert o.first_bad is not None
    assert s.last_error_cell() == o.first_bad
    s.clear_error_cell()
    assert s.last_error_cell() is None


def _negative_pressure_case(scheme):
    from hyperflow_gb300 import cases
    case = cases.quadrant_case(40, ny=36, scheme=scheme, limiter="MinBee", split=(0.45, 0.55))
    g = 1 if scheme == "Godunov" else 2
    return case, (g + 17, g + 23)   # interior cell (i 23, j 17)


@pytest.mark.parametrize("scheme", ["Godunov", "MUSCLHancock"])
def test_gpu_negative_pressure_cell_matches_oracle(scheme, port_lib):
    """A cell with negative total energy (pressure < 0, NaN sound speed): the NaNs, the
    zero-flux count and the earliest zero-flux face all match the oracle, step by step."""
    from oracle.oracle import Oracle
    case, (j, i) = _negative_pressure_case(scheme)
    o, s = Oracle(case), _solver(case)
    U = s.state(0)
    U[3, j, i] = -1.0
    s.set_state(0, U)
    o.U[0][...] = U
    dts_o = o.run(4)
    dts = [s.step() for _ in range(4)]
    np.testing.assert_array_equal(np.array(dts), dts_o)
    np.testing.assert_array_equal(s.state(0), o.state(0))
    assert s.hllc_errors() == o.hllc_errors > 0
    bad = s.last_error_cell()
    assert bad == o.first_bad
    assert bad["step"] == 0 and bad["dir"] == 0 and abs(bad["i"] - 23) <= 3   # next to cell (23, 17)
    assert s.last_nonpositive_cell() == o.first_nonpos
    assert o.first_nonpos["step"] == 0


def test_gpu_nonpositive_cell_matches_oracle():
    """A physical start that loses positivity: the shock-bubble at 128^2 under MUSCL-Hancock at
    CFL 0.8 (unstable for 2D flow) first leaves a cell with negative pressure at step 82, before
    any zero-flux face.  The earliest non-positive cell, the later zero-flux face and the state
    with its NaNs all match the oracle; clearing forgets both records."""
    from oracle.oracle import Oracle
    from hyperflow_gb300 import cases
    case = cases.shock_bubble_case(128, cfl=0.8)
    o, s = Oracle(case, nthreads=4), _solver(case)
    o.run(82)
    s.run(82)
    assert o.first_nonpos is None and s.last_nonpositive_cell() is None
    o.run(8)
    s.run(8)
    np.testing.assert_array_equal(s.state(0), o.state(0))
    assert o.first_nonpos == {"step": 82, "block": 0, "j": 82, "i": 45}
    assert s.last_nonpositive_cell() == o.first_nonpos
    assert s.last_error_cell() == o.first_bad
    s.clear_error_cell()
    assert s.last_nonpositive_cell() is None and s.last_error_cell() is None


def test_gpu_strict_mode_stops_at_the_nonpositive_step():
    """Strict mode on the same run: the step that left the non-positive cell (step 82) completes
    and the loop stops there, through the device loop and through the piecewise calls."""
    from hyperflow_gb300 import HyperFlowError, cases
    case = cases.shock_bubble_case(128, cfl=0.8)
    s, ref = _solver(case), _solver(case)
    ref.run(83)
    s.set_strict(True)
    with pytest.raises(HyperFlowError, match="non-positive density or pressure at step 82, block 0, cell"):
        s.run(200)
    assert s.time()[:2] == ref.time()[:2]
    np.testing.assert_array_equal(s.state(0), ref.state(0))
    with pytest.raises(HyperFlowError, match="non-positive"):
        s.step()
    assert s.time()[:2] == ref.time()[:2]


def test_gpu_strict_mode_stops_at_the_zero_flux_step():
    """Strict mode: the step that met the zero flux completes, the loop stops there and the
    calls raise; clearing the record lets one more step run; strict off runs on."""
    from hyperflow_gb300 import HyperFlowError
    case, (j, i) = _negative_pressure_case("MUSCLHancock")
    s, ref = _solver(case), _solver(case)
    U = s.state(0)
    U[3, j, i] = -1.0
    s.set_state(0, U)
    ref.set_state(0, U)
    ref.step()
    s.set_strict(True)
    with pytest.raises(HyperFlowError, match="zero flux"):
        s.run(5)
    assert s.time()[0] == ref.time()[0]          # exactly one step ran
    with pytest.raises(HyperFlowError, match="zero flux"):
        s.run(3)
    assert s.time()[0] == ref.time()[0]          # stopped
    s.clear_error_cell()
    with pytest.raises(HyperFlowError, match="zero flux"):
        s.run(3)
    ref.step()
    assert s.time()[0] == ref.time()[0]          # one more step, then stopped again
    s.set_strict(False)
    assert s.run(3) == 3


@pytest.mark.parametrize("limiter", ["MinBee", "VanLeer"])
def test_gpu_adaptor_call_sequence_matches_oracle(limiter, port_lib):
    """The reference-side adaptor's call sequence (hyperflow_gb300/adaptor/gpu_scheme.h): per
    step the host applies the boundary conditions, every block's fields are uploaded in MeshBlock
    order [x][y][var] with ghosts, the device forms dt, and each block is advanced on the device
    and downloaded into the host fields -- bit for bit against the oracle's own step, dt included.
    The oracle stands in for the reference's host objects here; tests/test_adaptor.py compiles
    the adaptor itself against the reference's sources."""
    from hyperflow_gb300 import cases
    from oracle.oracle import Oracle
    case = cases.forward_facing_step_case(20, limiter=limiter)
    ref, host = Oracle(case), Oracle(case)
    s = _solver(case)
    for _ in range(12):
        dt_ref = float(ref.run(1)[0])
        host.apply_bcs()                                        # Mesh::apply_bcs on the host
        for b in range(s.nblocks):
            s.set_state(b, host.U[b].transpose(2, 1, 0), layout="aos")
        dt = s.calculate_time_step()                            # GpuScheme::calculate_time_step
        assert dt == dt_ref
        for b in range(s.nblocks):                              # GpuForwardEuler, block by block
            s.advance_block(b, dt)
            host.U[b][...] = s.state(b, layout="aos").transpose(2, 1, 0)
    for b in range(s.nblocks):
        np.testing.assert_array_equal(host.U[b], ref.state(b))


@pytest.mark.parametrize("scheme", ["Godunov", "MUSCLHancock"])
@pytest.mark.parametrize("upload", [False, True])
def test_gpu_fixed_dt_steps_without_time_step_match_oracle(scheme, upload, port_lib):
    """A caller that gives dt itself and never calls TimeStep: ghost fill (on the device, or on
    the host and uploaded), then every block advanced.  The MUSCL-Hancock predictor still makes
    its own TimeStep call over all cells, ghosts included -- here the Dirichlet inflow ghosts are
    the fastest cells (Mach 3 inflow into a slower start), so their maxima must be current."""
    from hyperflow_gb300 import cases
    from oracle.oracle import Oracle
    case = cases.forward_facing_step_case(20, scheme=scheme) if scheme == "Godunov" else \
        cases.forward_facing_step_case(20, limiter="VanLeer")
    case["initial_condition"]["init_state"] = [1.4, 0.5, 0.0, 1.0]
    o, host, s = Oracle(case), Oracle(case), _solver(case)
    for k in range(10):
        dt = 2e-3 if k < 5 else 4e-3
        o.apply_bcs()
        o.advance(dt)
        if upload:
            host.apply_bcs()
            for b in range(s.nblocks):
                s.set_state(b, host.U[b])
        else:
            s.apply_bcs()
        s.advance(dt)
        if upload:
            for b in range(s.nblocks):
                host.U[b][...] = s.state(b)
    for b in range(s.nblocks):
        np.testing.assert_array_equal(s.state(b), o.state(b))
    assert s.time()[1] == o.calls


def test_gpu_interleaved_contexts_are_independent():
    """Two contexts of different cases and schemes stepped in turn, in one process and on one
    device (the device loop, the piecewise calls, the host-buffer step), each equal to the same
    case run alone."""
    import threading
    from hyperflow_gb300 import cases
    ca = cases.forward_facing_step_case(20, limiter="MinBee")
    cb = cases.quadrant_case(64, scheme="Godunov")
    a, b = _solver(ca), _solver(cb)
    for k in range(6):
        a.run(2)
        b.apply_bcs()
        b.advance(b.calculate_time_step())
        host = [a.state(i) for i in range(a.nblocks)]
        a.step_io(host)
        b.run(1, graph=False)
    a0, b0 = _solver(ca), _solver(cb)
    a0.run(18)
    b0.run(12)
    for i in range(a.nblocks):
        np.testing.assert_array_equal(a.state(i), a0.state(i))
    np.testing.assert_array_equal(b.state(0), b0.state(0))
    # two host threads, one context each
    a1, b1 = _solver(ca), _solver(cb)
    t = [threading.Thread(target=a1.run, args=(18,)), threading.Thread(target=b1.run, args=(12,))]
    for x in t:
        x.start()
    for x in t:
        x.join()
    for i in range(a.nblocks):
        np.testing.assert_array_equal(a1.state(i), a0.state(i))
    np.testing.assert_array_equal(b1.state(0), b0.state(0))


def test_gpu_piecewise_api_equals_device_loop():
    """apply_bcs / calculate_time_step / advance_block driven from the host (the
    reference's Simulation::solve sequence) equals hf_run's device loop, with and
    without the CUDA graph."""
    from hyperflow_gb300 import cases
    case = cases.forward_facing_step_case(40, limiter="MinBee")
    a, b, c = _solver(case), _solver(case), _solver(case)
    for _ in range(25):
        a.apply_bcs()
        dt = a.calculate_time_step()
        for blk in range(a.nblocks):
            a.advance_block(blk, dt)
    b.run(25, graph=True)
    c.run(25, graph=False)
    for blk in range(3):
        np.testing.assert_array_equal(a.state(blk), b.state(blk))
        np.testing.assert_array_equal(a.state(blk), c.state(blk))
    assert a.time()[:2] == b.time()[:2] == c.time()[:2]


def test_gpu_state_layouts_round_trip():
    from hyperflow_gb300 import cases
    s = _solver(cases.quadrant_case(20, ny=13, scheme="MUSCLHancock", limiter="MinBee"))
    s.run(3)
    soa = s.state(0)
    aos = s.state(0, layout="aos")
    np.testing.assert_array_equal(np.transpose(aos, (2, 1, 0)), soa)
    s.set_state(0, aos, layout="aos")
    np.testing.assert_array_equal(s.state(0), soa)


def test_gpu_set_state_then_step_matches_oracle(port_lib):
    """An uploaded arbitrary state (a drop-in caller's fields) steps exactly like the
    reference: the interior TimeStep terms are recomputed from the upload."""
    from hyperflow_gb300 import cases
    from oracle.oracle import Oracle
    case = cases.quadrant_case(36, ny=28, scheme="MUSCLHancock", limiter="VanLeer")
    rng = np.random.default_rng(5)
    o = Oracle(case)
    U = o.state(0)
    g = 2
    U[0, g:-g, g:-g] *= rng.uniform(0.8, 1.2, U[0, g:-g, g:-g].shape)
    U[3, g:-g, g:-g] *= rng.uniform(0.9, 1.1, U[3, g:-g, g:-g].shape)
    o.set_state(0, U)
    s = _solver(case)
    s.set_state(0, U)
    o.run(15)
    s.run(15)
    np.testing.assert_array_equal(s.state(0), o.state(0))


@pytest.mark.parametrize("which", ["godunov_256", "mh_minbee_ffs_full", "mh_vanleer_ffs_full", "mh_vanleer_4096"])
def test_gpu_full_size_matches_oracle(which, port_lib):
    """The full benchmark sizes against the oracle on all host cores: the 256^2 Godunov workload
    to its 200 steps; the 4.7M-cell forward-facing step (dx = 1/1365, the benchmark's workload)
    for 200 steps with each limiter -- ten times the benchmark's timed steps, past the start-up
    factor's 10 TimeStep calls; its full run to t = 4 at dx = 1/40 is the reference's own
    fixture (cart_ffs_*_dx1_40_t4); and 4096^2 MUSCL-Hancock for 2 steps."""
    import os
    from hyperflow_gb300 import cases
    from oracle.oracle import Oracle
    if which == "godunov_256":
        case, steps = cases.quadrant_case(256), 200
    elif which == "mh_minbee_ffs_full":
        case, steps = cases.forward_facing_step_case(1365, limiter="MinBee"), 200
    elif which == "mh_vanleer_ffs_full":
        case, steps = cases.forward_facing_step_case(1365, limiter="VanLeer"), 200
    else:
        case, steps = cases.quadrant_case(4096, scheme="MUSCLHancock", limiter="VanLeer"), 2
    o = Oracle(case, nthreads=os.cpu_count() or 4)
    o.run(steps)
    s = _solver(case)
    s.run(steps)
    for b in range(s.nblocks):
        np.testing.assert_array_equal(s.state(b), o.state(b))
    assert s.time()[1] == o.calls


def test_gpu_reflective_box_conserves_mass():
    """Closed reflective box, Godunov: the wall mass flux of HLLC between mirror states
    is zero to rounding, so total mass is conserved to round-off over many steps (a
    size-independent property at a large size).  MUSCL-Hancock is not held to this:
    the reference's slope clamp maps a zero difference to +1e-6 whatever its side
    (muscl_hancock.cpp:78-84), so ghost and interior slopes are not exact mirrors and
    the wall leaks mass at the 1e-7 level -- in the reference as well."""
    from hyperflow_gb300 import cases
    case = cases.quadrant_case(1024, bc="Reflective")
    s = _solver(case)
    g = 1
    m0 = math.fsum(s.state(0)[0, g:-g, g:-g].ravel())
    s.run(200)
    m1 = math.fsum(s.state(0)[0, g:-g, g:-g].ravel())
    assert abs(m1 - m0) <= 1e-12 * abs(m0)


def test_gpu_transpose_symmetry():
    """x<->y mirrored initial data gives the transposed solution (to rounding: the
    reference's x and y fluxes group products differently, e.g. (rho*u)*v)."""
    from hyperflow_gb300 import cases
    st = ([1.0, 0.0, 0.0, 1.0], [0.5, 0.3, 0.1, 0.4], [0.2, 0.2, 0.2, 0.1], [0.5, 0.1, 0.3, 0.4])
    a = _solver(cases.quadrant_case(128, scheme="MUSCLHancock", limiter="VanLeer", states=st))
    a.run(60)
    Ua = a.state(0)
    sym = np.stack([Ua[0].T, Ua[2].T, Ua[1].T, Ua[3].T])
    # rounding asymmetry grows through limiter switches (~1e-8 after 60 steps); an x/y
    # mix-up in a kernel would show at O(1)
    np.testing.assert_allclose(Ua, sym, rtol=1e-6, atol=1e-9)


def test_gpu_shock_bubble_matches_oracle(port_lib):
    """The shock-bubble initial condition (no reference counterpart) on the GPU path and in
    the oracle, 512^2 MUSCL-Hancock, bit for bit."""
    from hyperflow_gb300 import cases
    from oracle.oracle import Oracle
    case = cases.shock_bubble_case(512)
    o = Oracle(case, nthreads=8)
    s = _solver(case)
    np.testing.assert_array_equal(s.state(0), o.state(0))
    o.run(40)
    s.run(40)
    np.testing.assert_array_equal(s.state(0), o.state(0))


def _host_arrays(like, memory):
    if memory == "pageable":
        return [x.copy() for x in like]
    import torch
    out = []
    for x in like:
        t = torch.empty(x.shape, dtype=torch.float64).pin_memory()
        a = t.numpy()
        a[...] = x
        out.append(a)              # the array's base keeps the pinned tensor alive
    return out


@pytest.mark.parametrize("memory", ["pageable", "pinned", "pinned-separate-out"])
@pytest.mark.parametrize("scheme", ["Godunov", "MUSCLHancock"])
def test_gpu_step_io_equals_upload_step_download(memory, scheme):
    """hf_step_io against hf_set_state + hf_step + hf_get_state on the 3-block forward-facing
    step, several steps in a row: pageable arrays take the copy path (overlapped per-block
    downloads); pinned arrays the direct path (the kernels read the host arrays and the
    stencils store their cells to them), in place and into separate output arrays."""
    from hyperflow_gb300 import CartSolver, cases
    case = cases.forward_facing_step_case(40, scheme="Godunov") if scheme == "Godunov" else \
        cases.forward_facing_step_case(40, limiter="VanLeer")
    a, b = _solver(case), _solver(case)
    a.run(5)
    b.run(5)                       # the same TimeStep call count (it sets the CFL factor)
    host = _host_arrays([a.state(k) for k in range(a.nblocks)], memory.split("-")[0])
    outs = None
    if memory == "pinned-separate-out":
        outs = _host_arrays([np.full_like(x, np.nan) for x in host], "pinned")
    for x in host + (outs or []):
        assert CartSolver.host_mapped(x) == memory.startswith("pinned")
    for _ in range(4):
        for k in range(b.nblocks):
            b.set_state(k, host[k])
        dt_b = b.step()
        want = [b.state(k) for k in range(b.nblocks)]
        dt_a = a.step_io(host, outs)
        assert dt_a == dt_b
        for k in range(a.nblocks):
            np.testing.assert_array_equal((outs or host)[k], want[k])
            np.testing.assert_array_equal(a.state(k), want[k])
        if outs is not None:
            for k in range(a.nblocks):
                host[k][...] = outs[k]
                outs[k][...] = np.nan


@pytest.mark.parametrize("scheme,limiter", [("Godunov", None), ("MUSCLHancock", "MinBee"),
                                            ("MUSCLHancock", "VanLeer")])
@pytest.mark.parametrize("nx,ny", [(1, 1), (1, 5), (3, 2), (33, 1), (33, 13), (65, 25), (33, 11), (65, 21),
                                   (31, 43)])
def test_gpu_tiny_and_ragged_grids_match_oracle(scheme, limiter, nx, ny, port_lib):
    """Grids smaller than one tile, and one cell past a tile edge in x and y (MUSCL-Hancock
    tiles 32x12, Godunov 32x10): partial tiles and clipped faces.  Blocks narrower than 2 x ghost cells (the ghost
    fill would mirror ghost cells into ghost cells, in the reference's sequential order) are
    refused with HF_ERR_UNSUPPORTED instead of computed."""
    from oracle.oracle import Oracle
    from hyperflow_gb300 import HyperFlowError, cases
    case = cases.quadrant_case(nx, ny=ny, scheme=scheme, limiter=limiter, split=(0.45, 0.55))
    g = 1 if scheme == "Godunov" else 2
    if nx < 2 * g or ny < 2 * g:
        with pytest.raises(HyperFlowError, match="2\\*ghost"):
            _solver(case)
        return
    o = Oracle(case)
    s = _solver(case)
    dts_o = o.run(25)
    dts = [s.step() for _ in range(25)]
    np.testing.assert_array_equal(np.array(dts), dts_o)
    np.testing.assert_array_equal(s.state(0), o.state(0))
    assert s.hllc_errors() == o.hllc_errors


def _fast_block0(case, seed=3):
    """the forward-facing step with block 0's interior replaced by a seeded field whose waves
    are the fastest of the mesh and change every step"""
    from oracle.oracle import Oracle
    o = Oracle(case)
    U = o.state(0)
    rng = np.random.default_rng(seed)
    g = 2
    inner = (slice(None), slice(g, -g), slice(g, -g))
    shape = U[inner][0].shape
    rho = rng.uniform(0.5, 2.0, shape)
    u = rng.uniform(2.0, 6.0, shape)
    v = rng.uniform(-1.0, 1.0, shape)
    p = rng.uniform(0.5, 3.0, shape)
    W = np.stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)])
    U[inner] = W
    return U


@pytest.mark.parametrize("limiter", ["MinBee", "VanLeer"])
def test_gpu_all_blocks_launch_reruns_a_block_whose_predictor_dt_changed(limiter, port_lib):
    """The all-blocks launch runs every block with the predictor dt of the step's starting state
    and runs block b again when the reference's predictor dt (blocks < b updated) differs.  Here
    block 0 holds the fastest waves and they change every step, so blocks 1 and 2 are run twice
    in most steps: the results equal the oracle's bit for bit, as do those of the one-launch-per-
    block mode, and the re-run count is positive."""
    from hyperflow_gb300 import cases
    from oracle.oracle import Oracle
    case = cases.forward_facing_step_case(40, limiter=limiter)
    U0 = _fast_block0(case)
    o = Oracle(case)
    o.set_state(0, U0)
    o.run(12)
    for per_block in (False, True):
        s = _solver(case)
        s.set_block_launches(per_block)
        s.set_state(0, U0)
        s.run(7, graph=False)
        s.run(5, graph=True)
        for b in range(3):
            np.testing.assert_array_equal(s.state(b), o.state(b), err_msg=f"block {b}, per_block={per_block}")
        assert s.time()[1] == o.calls
        assert (s.blocks_rerun() > 0) == (not per_block)


def test_gpu_all_blocks_launch_equals_per_block_launches_on_the_benchmark_step(port_lib):
    """The 4.7M-cell forward-facing step for 30 steps in both launch modes: identical states,
    time and TimeStep calls."""
    from hyperflow_gb300 import cases
    case = cases.forward_facing_step_case(1365, limiter="MinBee")
    a, b = _solver(case), _solver(case)
    b.set_block_launches(True)
    a.run(30)
    b.run(30)
    assert a.time() == b.time()
    for k in range(3):
        np.testing.assert_array_equal(a.state(k), b.state(k))
    assert a.hllc_errors() == b.hllc_errors() == 0
