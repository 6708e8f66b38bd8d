"""Frame images (the reference's plotting script, euler_2d.py, headless): the schlieren oracle
against the reference's own method, the PNG writer, the domain-grid assembly of a multi-block
frame, and -- on the GPU -- the image kernel against the oracle."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _golden():
    return np.load(os.path.join(GOLDEN, "render_schlieren.npz"))


def test_schlieren_oracle_matches_reference_method():
    from oracle.render_oracle import schlieren
    g = _golden()
    for k in range(3):
        ours = schlieren(g[f"in{k}"], float(g[f"dx{k}"]), float(g[f"dy{k}"]))
        ref = g[f"out{k}"]
        assert np.array_equal(np.isnan(ours), np.isnan(ref))
        np.testing.assert_allclose(ours, ref, rtol=4e-16, atol=0)   # exp may differ by an ulp


def test_schlieren_oracle_edge_cases():
    from oracle.render_oracle import schlieren
    flat = schlieren(np.full((5, 4), 2.0), 0.1, 0.1)           # max |grad| = 0: 0/0 everywhere
    assert np.isnan(flat).all()
    tiny = schlieren(np.arange(4.0).reshape(2, 2), 0.1, 0.1)   # no interior cell: max stays -1e6
    np.testing.assert_array_equal(tiny, np.ones((2, 2)))


def test_png_round_trip(tmp_path):
    from hyperflow_gb300.render import read_png, write_png
    img = (np.arange(37 * 23) % 256).astype(np.uint8).reshape(23, 37)
    p = str(tmp_path / "a.png")
    write_png(p, img)
    with open(p, "rb") as fh:
        assert fh.read(8) == b"\x89PNG\r\n\x1a\n"
    np.testing.assert_array_equal(read_png(p), img)


def test_domain_grid_of_the_forward_facing_step():
    """Three blocks on one cell size: each lands at its extents, the step's corner stays NaN."""
    from hyperflow_gb300 import cases
    from hyperflow_gb300.frames import case_meta
    from hyperflow_gb300.render import domain_grid
    case = cases.forward_facing_step_case(20)
    meta = case_meta(case)
    rng = np.random.default_rng(0)
    blocks = [rng.uniform(1.0, 2.0, (4, b["ny"], b["nx"])) for b in meta["blocks"]]
    head = dict(meta, index=0, t=0.0)
    grid, dx, dy = domain_grid(head, blocks, "rho")
    assert grid.shape == (20, 60) and dx == pytest.approx(0.05) and dy == pytest.approx(0.05)
    np.testing.assert_array_equal(grid[0:4, 0:12], blocks[0][0])     # [0,0.6] x [0,0.2]
    np.testing.assert_array_equal(grid[4:20, 0:12], blocks[1][0])    # [0,0.6] x [0.2,1]
    np.testing.assert_array_equal(grid[4:20, 12:60], blocks[2][0])   # [0.6,3] x [0.2,1]
    assert np.isnan(grid[0:4, 12:60]).all()                          # the step
    p = domain_grid(head, blocks, "p")[0]
    r, ru, rv, E = blocks[0]
    u, v = ru / r, rv / r
    np.testing.assert_array_equal(p[0:4, 0:12], (1.4 - 1.0) * (E - 0.5 * r * (u * u + v * v)))


@pytest.mark.gpu
def test_gpu_schlieren_and_image_match_oracle():
    from oracle.render_oracle import grey, schlieren
    from hyperflow_gb300.render import render_grid
    g = _golden()
    for k in range(3):
        f = g[f"in{k}"]                        # [x][y]; the kernel takes [y][x]
        dx, dy = float(g[f"dx{k}"]), float(g[f"dy{k}"])
        field, img = render_grid(f.T.copy(), dx, dy, schlieren=True)
        ref = schlieren(f, dx, dy)
        assert np.array_equal(np.isnan(field.T), np.isnan(ref))
        np.testing.assert_allclose(field.T, ref, rtol=1e-15, atol=0)
        want = grey(ref.T)
        assert (np.abs(img.astype(int) - want.astype(int)) > 1).sum() == 0
        assert (img != want).mean() < 1e-3
        plain, pimg = render_grid(f.T.copy(), dx, dy, schlieren=False, limits=(0.0, 2.0))
        np.testing.assert_array_equal(plain, f.T)
        np.testing.assert_array_equal(pimg, grey(f.T, (0.0, 2.0)))


@pytest.mark.gpu
def test_gpu_render_frames_of_a_run(tmp_path):
    """solve() frames of the forward-facing step rendered to PNGs, one per frame, the density
    schlieren of the last equal to the oracle's image of the same frame."""
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300 import frames as fr
    from hyperflow_gb300.render import domain_grid, read_png, render_frames
    from oracle.render_oracle import grey, schlieren
    case = cases.forward_facing_step_case(20)
    case["simulation"]["t_end"] = 0.5
    case["simulation"]["animation"] = {"duration": 1.0, "fps": 4}
    s = CartSolver(case)
    s.solve(out_dir=str(tmp_path / "frames"))
    pngs = render_frames(str(tmp_path / "frames"), str(tmp_path / "png"), "rho-gradient")
    assert len(pngs) == len(s.frame_paths) >= 4
    head, blocks = fr.read_frame(sorted(s.frame_paths)[-1])
    grid, dx, dy = domain_grid(head, blocks, "rho")
    want = grey(schlieren(grid.T, dx, dy).T)[::-1]
    got = read_png(pngs[-1])
    assert got.shape == want.shape and (np.abs(got.astype(int) - want.astype(int)) > 1).sum() == 0
