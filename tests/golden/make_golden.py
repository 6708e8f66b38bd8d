"""Generates the golden fixtures in this folder from the reference solver itself.

Run where the reference tree exists (it builds oracle/_ref/ from the reference's own
sources with ``make -C oracle ref``):

    python tests/golden/make_golden.py

Each fixture is an .npz holding the case JSON, the number of steps, the reference's
step dt stream, every TimeStep call it made (step calls and MUSCL-Hancock predictor
calls), and the final state of every block (SoA [var][y][x], ghosts included) -- or,
for the full-size 256x256 Godunov workload, per-variable checksums and a seeded sample
of cells instead of the whole state.  Unit fixtures hold HLLC fluxes and limiter values
for random and edge-case inputs.  Frame fixtures hold what the reference's own
Simulation::solve writes (the hash of every CSV frame), its TimeStep calls and final state.
"""
from __future__ import annotations

import json
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hyperflow_gb300 import cases  # noqa: E402
from oracle import oracle, reference_root  # noqa: E402

REF_CASES = os.path.join(reference_root(), "cases", "fvm_2d_cart")

# (ne, nw, sw, se) primitive states of two rarefactions moving apart at speed 2 / 3
VACUUM2 = ([1.0, 2.0, 0.0, 0.4], [1.0, -2.0, 0.0, 0.4], [1.0, -2.0, 0.0, 0.4], [1.0, 2.0, 0.0, 0.4])
VACUUM3 = ([1.0, 3.0, 0.0, 0.4], [1.0, -3.0, 0.0, 0.4], [1.0, -3.0, 0.0, 0.4], [1.0, 3.0, 0.0, 0.4])


def cart_cases():
    """(name, case, steps, clamp_t_end, full_state)"""
    out = [
        ("godunov_quad_48", cases.quadrant_case(48), 60, False, True),
        ("godunov_quad_ragged_37x29", cases.quadrant_case(37, ny=29, split=(0.41, 0.63)), 50, False, True),
        ("godunov_quad_reflective_40", cases.quadrant_case(40, bc="Reflective"), 60, False, True),
        ("mh_minbee_quad_48", cases.quadrant_case(48, scheme="MUSCLHancock", limiter="MinBee"), 60, False, True),
        ("mh_vanleer_quad_44x36", cases.quadrant_case(44, ny=36, scheme="MUSCLHancock", limiter="VanLeer"), 60, False, True),
        ("mh_minbee_reflective_33x47", cases.quadrant_case(33, ny=47, scheme="MUSCLHancock", limiter="MinBee",
                                                           bc="Reflective", split=(0.55, 0.35)), 50, False, True),
        ("ffs_minbee_dx1_40", cases.forward_facing_step_case(40, limiter="MinBee"), 60, False, True),
        ("ffs_vanleer_dx1_40", cases.forward_facing_step_case(40, limiter="VanLeer"), 60, False, True),
        ("ffs_godunov_dx1_30", cases.forward_facing_step_case(30, scheme="Godunov"), 60, False, True),
        # double rarefaction towards vacuum: the reference's HLLC "should not get here"
        # zero-flux branch (riemann_hllc.cpp:207-211) fires hundreds of times per step
        ("mh_minbee_vacuum_hllc_fallback", cases.quadrant_case(
            32, ny=24, scheme="MUSCLHancock", limiter="MinBee", states=VACUUM2), 20, False, True),
        ("mh_vanleer_vacuum_hllc_fallback", cases.quadrant_case(
            30, ny=26, scheme="MUSCLHancock", limiter="VanLeer", states=VACUUM3), 20, False, True),
        # the 256x256 Godunov workload at full length
        ("godunov_quad_256_200", cases.quadrant_case(256), 200, False, False),
        # the forward-facing step to its end time t = 4 (about 800 steps) at dx = 1/40
        ("ffs_minbee_dx1_40_t4", cases.forward_facing_step_case(40, limiter="MinBee"), 10**6, True, True),
        ("ffs_vanleer_dx1_40_t4", cases.forward_facing_step_case(40, limiter="VanLeer"), 10**6, True, True),
    ]
    for rel, steps in [("shock_tubes/toro/toro_shock_tube_01_godunov_hllc_100x5.json", 400),
                       ("shock_tubes/toro/toro_shock_tube_01_muscl_hancock_vanleer_hllc_100x5.json", 400),
                       ("sphericalrp/sphericalrp_godunov_hllc_50x50.json", 120),
                       ("sphericalrp/sphericalrp_muscl_hancock_vanleer_hllc_50x50.json", 120)]:
        with open(os.path.join(REF_CASES, rel)) as f:
            case = json.load(f)
        name = "refcase_" + os.path.splitext(os.path.basename(rel))[0]
        out.append((name, case, steps, True, True))
    return out


def sample_idx(shape, n=2000, seed=7):
    rng = np.random.default_rng(seed)
    return np.stack([rng.integers(0, s, n) for s in shape[1:]], axis=0)


def make_cart(only=None):
    for name, case, steps, clamp, full in cart_cases():
        if only and name not in only:
            continue
        ref = oracle.RefCart(case)
        taken = ref.run(steps, clamp)
        blocks = [ref.state(b) for b in range(ref.nblocks())]
        data = {"case": json.dumps(case), "steps": taken, "clamp": int(clamp),
                "step_dts": ref.step_dts(), "calls": ref.calls(), "t": ref.time(),
                "nblocks": len(blocks)}
        if full:
            for b, U in enumerate(blocks):
                data[f"U{b}"] = U
        else:
            U = blocks[0]
            idx = sample_idx(U.shape)
            data["sample_idx"] = idx
            data["sample"] = U[:, idx[0], idx[1]]
            data["sums"] = np.array([math.fsum(U[v].ravel()) for v in range(4)])
            data["sumsq"] = np.array([math.fsum((U[v] * U[v]).ravel()) for v in range(4)])
        np.savez_compressed(os.path.join(HERE, f"cart_{name}.npz"), **data)
        print(name, taken, "steps")


FRAME_CASES = ["shock_tubes/toro/toro_shock_tube_01_godunov_hllc_100x5.json",
               "shock_tubes/toro/toro_shock_tube_01_muscl_hancock_vanleer_hllc_100x5.json",
               "sphericalrp/sphericalrp_godunov_hllc_50x50.json"]


def make_frames():
    """The reference's own Simulation::solve with its frame output: the sha256 of every CSV
    frame it writes (results_%06d.csv), its TimeStep call stream and its final state."""
    import hashlib
    import tempfile
    for rel in FRAME_CASES:
        with open(os.path.join(REF_CASES, rel)) as f:
            case = json.load(f)
        name = os.path.splitext(os.path.basename(rel))[0]
        ref = oracle.RefCart(case)
        with tempfile.TemporaryDirectory() as d:
            ref.solve(d)
            files = sorted(os.listdir(d))
            hashes = [hashlib.sha256(open(os.path.join(d, fn), "rb").read()).hexdigest() for fn in files]
        data = {"case": json.dumps(case), "csv_sha256": np.array(hashes), "calls": ref.calls(),
                "nblocks": ref.nblocks()}
        for b in range(ref.nblocks()):
            data[f"U{b}"] = ref.state(b)
        np.savez_compressed(os.path.join(HERE, f"frames_{name}.npz"), **data)
        print(name, len(files), "frames")


def make_uns_frames():
    """The reference's own unstructured Simulation::solve with frame output."""
    import hashlib
    import tempfile
    from hyperflow_gb300 import meshgen
    sets = [("quad_channel_240", *quad_channel(), 0.05, 20.0),
            ("tri_hole_3k", *meshgen.jittered_hole_mesh(3000, seed=3), 0.02, 10.0)]
    for name, verts, codes, t_end, fps in sets:
        nbr = oracle.ref_neighbours(verts, codes)[0]
        case = meshgen.channel_case("mesh.hmsh", cfl=0.5, t_end=t_end)
        case["simulation"]["animation"] = {"duration": 1.0, "fps": fps}
        nverts = np.full(len(verts), verts.shape[1], np.int32)
        ref = oracle.RefUns(case, nverts, verts.reshape(-1, 2), nbr)
        cen = ref.centroids()
        with tempfile.TemporaryDirectory() as d:
            ref.solve(d)
            files = sorted(os.listdir(d))
            hashes = [hashlib.sha256(open(os.path.join(d, fn), "rb").read()).hexdigest() for fn in files]
        np.savez_compressed(os.path.join(HERE, f"unsframes_{name}.npz"), case=json.dumps(case),
                            verts=verts, codes=codes, nbr=nbr, centroids=cen,
                            csv_sha256=np.array(hashes), U=ref.state())
        print("uns frames", name, len(files), "frames")


def unit_states(n=4000, seed=11):
    """Random conservative states plus hand-picked edge cases (vacuum-like, supersonic,
    zero velocity, equal states, NaN/inf)."""
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.uniform(np.log(1e-3), np.log(10.0), n))
    u = rng.uniform(-5, 5, n)
    v = rng.uniform(-5, 5, n)
    p = np.exp(rng.uniform(np.log(1e-4), np.log(100.0), n))
    W = np.stack([rho, u, v, p], 1)
    W[::17, 1] = 0.0
    W[::23, 2] = 0.0
    W[::29, 1] *= 40.0     # strongly supersonic
    U = np.stack([oracle.prim_to_cons(w) for w in W])
    return U


def make_units():
    lib = oracle.ref_cart_lib()
    UL = unit_states(4000, 11)
    UR = unit_states(4000, 12)
    UR[::31] = UL[::31]                        # identical states
    UL[5] = [np.nan, 0, 0, 1]                  # NaN density
    UR[6] = [1.0, np.inf, 0.0, 1.0]            # infinite momentum
    UL[7] = [1.0, 0.0, 0.0, -1.0]              # negative energy -> NaN sound speed
    UL[8] = [0.0, 0.0, 0.0, 0.0]               # vacuum
    F = np.zeros((2, len(UL), 4))
    for d in range(2):
        for k in range(len(UL)):
            f = np.zeros(4)
            a = np.ascontiguousarray(UL[k])
            b = np.ascontiguousarray(UR[k])
            lib.hfref_hllc(1.4, a.ctypes.data, b.ctypes.data, d, f.ctypes.data)
            F[d, k] = f
    rng = np.random.default_rng(3)
    r = np.concatenate([rng.uniform(-3, 5, 3000), np.exp(rng.uniform(-20, 20, 500)),
                        [0.0, -0.0, 1.0, 1.0 + 2**-52, 1.0 - 2**-53, -1.0, -1.0 + 1e-7,
                         -1.0 - 1e-7, -0.9999999, np.inf, -np.inf, np.nan, 1e-300, -1e-300,
                         2.0, 3.0, 0.5]])
    lim = np.array([[lib.hfref_limiter(k, float(x)) for x in r] for k in range(2)])
    np.savez_compressed(os.path.join(HERE, "unit_hllc_limiter.npz"), UL=UL, UR=UR, F=F, r=r, lim=lim)
    print("units", len(UL), len(r))


def quad_channel(nx=24, ny=10, seed=4):
    """A quadrilateral channel mesh in the reference's quad format: jittered interior
    vertices, inlet on the left, transmissive right, reflective top and bottom."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 2.4, nx + 1)
    ys = np.linspace(0.0, 1.0, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    inner = (slice(1, nx), slice(1, ny))
    X[inner] += rng.uniform(-0.2, 0.2, X[inner].shape) * (xs[1] - xs[0])
    Y[inner] += rng.uniform(-0.2, 0.2, Y[inner].shape) * (ys[1] - ys[0])
    verts, codes = [], []
    for i in range(nx):
        for j in range(ny):
            v = [(X[i, j], Y[i, j]), (X[i + 1, j], Y[i + 1, j]), (X[i + 1, j + 1], Y[i + 1, j + 1]),
                 (X[i, j + 1], Y[i, j + 1])]
            verts.append(v)
            # edges: bottom, right, top, left
            codes.append([-1 if j == 0 else 0, -2 if i == nx - 1 else 0, -1 if j == ny - 1 else 0,
                          -3 if i == 0 else 0])
    return np.array(verts, dtype=np.float64), np.array(codes, dtype=np.int32)


def _ref_uns(case, verts, codes, tmpdir):
    """The reference's unstructured solver on this mesh, and the neighbours it used.  Quad
    meshes go through the reference's own loader (the mesh written to a file, read by
    LoadStructuredMesh with its O(E^2) tolerance search); triangle meshes, which that loader
    cannot read, take the oracle's restatement of the same search (pinned against the loader on
    the quad meshes)."""
    from hyperflow_gb300 import meshgen
    if verts.shape[1] == 4:
        path = os.path.join(tmpdir, "mesh.hmsh")
        with open(path, "w") as f:
            f.write(meshgen.hmsh_text(verts, codes))
        fcase = json.loads(json.dumps(case))
        fcase["mesh"]["file"] = path
        fcase["mesh"]["type"] = "hyperflow_structured"   # the one type parser.cpp:146 reads
        ref = oracle.RefUns.from_file(fcase)
        return ref, ref.nbr.copy()
    nbr = oracle.ref_neighbours(verts, codes)[0]
    nverts = np.full(len(verts), verts.shape[1], np.int32)
    return oracle.RefUns(case, nverts, verts.reshape(-1, 2), nbr), nbr


def scramjet(reduction: int):
    """The reference's own scramjet case (cases/fvm_2d_uns/scramjet_kumar): its block spec
    (scramjet_kumar_coarse_mesh.json, 17 blocks, 22,960 quads) with every block's cell counts
    divided by `reduction` (at least one cell), meshed by the reference's own
    src/mesh_generation/generate_block_mesh.py, and its case file
    (scramjet_kumar_godunov_hllc.json: Godunov + HLLC, CFL 0.5, Mach 5 inlet).  Blocks of that
    generator meet with vertex coordinates that differ in their last bits, so its neighbour
    search needs the reference loader's 1e-12 tolerance.  Returns (verts, codes, case)."""
    import importlib.util
    import tempfile
    from hyperflow_gb300 import meshgen
    ref = reference_root()
    spec = importlib.util.spec_from_file_location(
        "ref_generate_block_mesh", os.path.join(ref, "src", "mesh_generation", "generate_block_mesh.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    sdir = os.path.join(ref, "cases", "fvm_2d_uns", "scramjet_kumar")
    with open(os.path.join(sdir, "scramjet_kumar_coarse_mesh.json")) as f:
        blocks = json.load(f)
    for b in blocks:
        b["cells"] = [max(1, b["cells"][0] // reduction), max(1, b["cells"][1] // reduction)]
    with tempfile.TemporaryDirectory() as d:
        sp, mp = os.path.join(d, "blocks.json"), os.path.join(d, "mesh.hmsh")
        with open(sp, "w") as f:
            json.dump(blocks, f)
        gen.BlockStructuredMeshGenerator(sp).generate_mesh(mp)
        with open(mp) as f:
            verts, codes = meshgen.read_hmsh(f.read())
    with open(os.path.join(sdir, "scramjet_kumar_godunov_hllc.json")) as f:
        case = json.load(f)
    case["mesh"]["file"] = "mesh.hmsh"
    return np.array(verts, dtype=np.float64), np.array(codes, dtype=np.int32), case


def make_uns():
    import tempfile
    from hyperflow_gb300 import meshgen
    sets = [("tri_hole_3k", *meshgen.jittered_hole_mesh(3000, seed=3), meshgen.channel_case("mesh.hmsh", cfl=0.5), 40),
            ("quad_channel_240", *quad_channel(), meshgen.channel_case("mesh.hmsh", cfl=0.5), 60),
            ("scramjet_reduced4", *scramjet(4), 300)]
    for name, verts, codes, case, steps in sets:
        with tempfile.TemporaryDirectory() as d:
            ref, nbr = _ref_uns(case, verts, codes, d)
        ang, ln, area, rin = ref.geometry()
        ref.run(steps)
        np.savez_compressed(os.path.join(HERE, f"uns_{name}.npz"), case=json.dumps(case),
                            verts=verts, codes=codes, nbr=nbr, steps=steps, dts=ref.dts(),
                            U=ref.state(), angle=ang, length=ln, area=area, rin=rin)
        print("uns", name, len(verts), "cells", steps, "steps")


def make_loader():
    """The reference loader's neighbours on the full scramjet coarse mesh (22,960 quads,
    91,840 pairs; its O(E^2) scan takes about ten minutes)."""
    import tempfile
    verts, codes, case = scramjet(1)
    with tempfile.TemporaryDirectory() as d:
        ref, nbr = _ref_uns(case, verts, codes, d)
    np.savez_compressed(os.path.join(HERE, "loader_scramjet_coarse.npz"), verts=verts,
                        codes=codes.astype(np.int8), nbr=nbr)
    print("loader scramjet coarse", len(verts), "cells", len(nbr), "pairs")


if __name__ == "__main__":
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    which = sys.argv[1:] or ["units", "cart", "uns", "frames", "unsframes", "loader"]
    if "units" in which:
        make_units()
    if "cart" in which:
        make_cart()
    for w in which:
        if w.startswith("cart:"):      # cart:<fixture name>[,<name>...]
            make_cart(w[5:].split(","))
    if "uns" in which:
        make_uns()
    if "frames" in which:
        make_frames()
    if "unsframes" in which:
        make_uns_frames()
    if "loader" in which:
        make_loader()
