"""Frame output and its file formats on the CPU: the oracle's Simulation::solve cadence
(frame dt clamp, frame points and labels) against what the reference's own solve wrote
(golden hashes of its CSV frames, its TimeStep calls and final state), and the binary frame
file / CSV writer round trip."""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def frame_fixtures():
    return sorted(os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(GOLDEN, "frames_*.npz")))


def load_frames(name):
    d = np.load(os.path.join(GOLDEN, f"frames_{name}.npz"))
    out = {k: d[k] for k in d.files}
    out["case"] = json.loads(str(out["case"]))
    return out


def csv_hashes(case, labels, frames, every=1):
    from hyperflow_gb300 import frames as fr
    meta = fr.case_meta(case)
    return [hashlib.sha256(fr.csv_text(dict(meta, t=float(labels[k])), frames[k]).encode()).hexdigest()
            if k % every == 0 or k == len(frames) - 1 else None for k in range(len(frames))]


@pytest.mark.parametrize("name", frame_fixtures())
def test_oracle_solve_writes_the_reference_frames(name, port_lib):
    from oracle.oracle import Oracle
    g = load_frames(name)
    o = Oracle(g["case"])
    dts, labels, frames = o.solve(max_frames=len(g["csv_sha256"]) + 1)
    assert len(frames) == len(g["csv_sha256"])
    np.testing.assert_array_equal(np.array(o.calls), len(g["calls"]))
    for b in range(int(g["nblocks"])):
        np.testing.assert_array_equal(o.state(b), g[f"U{b}"])
    every = 1 if len(frames) < 100 else 37
    got = csv_hashes(g["case"], labels, frames, every)
    for k, h in enumerate(got):
        if h is not None:
            assert h == g["csv_sha256"][k], f"frame {k}"


def test_frame_file_round_trip_and_csv(tmp_path):
    from hyperflow_gb300 import cases, frames as fr
    case = cases.forward_facing_step_case(20)
    meta = fr.case_meta(case)
    rng = np.random.default_rng(0)
    blocks = [rng.random((4, b["ny"], b["nx"])) + 0.5 for b in meta["blocks"]]
    p = str(tmp_path / "results_000003.hfb")
    fr.write_frame(p, meta, 3, 0.125, blocks)
    head, got = fr.read_frame(p)
    assert head["index"] == 3 and head["t"] == 0.125 and head["blocks"] == meta["blocks"]
    for a, b in zip(blocks, got):
        np.testing.assert_array_equal(a, b)
    fr.to_csv(p, str(tmp_path / "f.csv"))
    text = open(tmp_path / "f.csv").read()
    assert text == fr.csv_text(head, blocks)
    lines = text.splitlines()
    assert lines[6] == "T=0.125" and lines[8] == "x,y,rho,rho_u,rho_v,E,u,v,p"
    assert len(lines) == 9 + sum(b["nx"] * b["ny"] for b in meta["blocks"])
    with pytest.raises(ValueError):
        open(tmp_path / "bad.hfb", "wb").write(b"not a frame")
        fr.read_frame(str(tmp_path / "bad.hfb"))


def test_frame_writer_thread(tmp_path):
    from hyperflow_gb300 import cases, frames as fr
    case = cases.quadrant_case(12)
    meta = fr.case_meta(case)
    w = fr.FrameWriter(str(tmp_path), meta, "hfb")
    for k in range(5):
        w.put(k, 0.1 * k, [np.full((4, 12, 12), float(k))])
    paths = w.close()
    assert [os.path.basename(p) for p in paths] == [f"results_{k:06d}.hfb" for k in range(5)]
    head, blocks = fr.read_frame(paths[4])
    assert head["t"] == 0.4 and blocks[0][2, 3, 4] == 4.0


def uns_frame_fixtures():
    return sorted(os.path.basename(p)[10:-4] for p in glob.glob(os.path.join(GOLDEN, "unsframes_*.npz")))


def load_uns_frames(name):
    d = np.load(os.path.join(GOLDEN, f"unsframes_{name}.npz"))
    out = {k: d[k] for k in d.files}
    out["case"] = json.loads(str(out["case"]))
    return out


def uns_oracle_solve(g):
    from oracle import oracle
    from hyperflow_gb300 import meshgen  # noqa: F401
    verts = g["verts"]
    nverts = np.full(len(verts), verts.shape[1], np.int32)
    ang, ln, area, rin = oracle.uns_geometry(nverts, verts.reshape(-1, 2))
    ps = np.concatenate([[0], np.cumsum(nverts)]).astype(np.int32)
    case = g["case"]
    gam = float(case["model"]["gamma"])
    inlet = oracle.prim_to_cons(case["mesh"]["boundaries"]["inlet"], gam)
    ic = case["initial_condition"]
    U = np.repeat(oracle.prim_to_cons(ic["init_state"], gam)[:, None], len(verts), axis=1)
    sim = case["simulation"]
    interval = float(sim["t_end"]) / (float(sim["animation"]["duration"]) * float(sim["animation"]["fps"]))
    steps, calls, labels, frames = oracle.uns_solve(gam, float(sim["cfl"]), ps, g["nbr"].ravel(), ang, ln,
                                                    area, rin, inlet, U, float(sim["t_start"]),
                                                    float(sim["t_end"]), interval, max_frames=256)
    return U, labels, frames


@pytest.mark.parametrize("name", uns_frame_fixtures())
def test_oracle_uns_solve_writes_the_reference_frames(name, port_lib):
    from hyperflow_gb300 import frames as fr
    g = load_uns_frames(name)
    U, labels, frames = uns_oracle_solve(g)
    np.testing.assert_array_equal(U, g["U"])
    assert len(frames) == len(g["csv_sha256"])
    meta = fr.uns_case_meta(g["case"], U.shape[1])
    for k in range(len(frames)):
        text = fr.uns_csv_text(dict(meta, t=float(labels[k])), frames[k], g["centroids"])
        assert hashlib.sha256(text.encode()).hexdigest() == g["csv_sha256"][k], k
