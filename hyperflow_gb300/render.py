"""Frame images, headless: the reference's plotting script (src/visualisation/euler/euler_2d.py)
for this package's binary frames.

The reference reads each CSV frame, pivots it onto the domain's cell grid (cells no block covers
stay NaN), and shows rho, u, v or p, or the "schlieren-like" normalised exponentiated gradient of
one of them ("rho-gradient", ...; euler_2d.py:214-295), with matplotlib.  Here the grid is
assembled from the full-precision frame (`frames.read_frame`), the field and an 8-bit grey image
are formed on the GPU (`hf_render_gray`), and the image is written as a PNG with the standard
library (grey levels: matplotlib and its colour maps are not part of this package).  Output files
are frame_%06d.png, as the reference names them.

    python -m hyperflow_gb300.render FRAMES_DIR OUT_DIR --var rho-gradient
"""
from __future__ import annotations

import argparse
import ctypes as C
import glob
import os
import struct
import zlib

import numpy as np

from . import frames as fr
from ._lib import check, lib

SCHLIEREN_BETA = 1.0      # euler_2d.py:185-186
SCHLIEREN_LAMBDA = 15.0
VARS = ("rho", "rho_u", "rho_v", "E", "u", "v", "p")


def cell_field(U: np.ndarray, var: str, gamma: float) -> np.ndarray:
    """One flow variable from a block's conservative state [4][ny][nx] (u, v, p as the CSV writer
    forms them, EulerIdealGasModel::cons_to_prim, euler_ideal_gas.cpp:76-92)."""
    r, ru, rv, E = U
    if var in ("rho", "rho_u", "rho_v", "E"):
        return {"rho": r, "rho_u": ru, "rho_v": rv, "E": E}[var]
    u = ru / r
    v = rv / r
    if var == "u":
        return u
    if var == "v":
        return v
    if var == "p":
        return (gamma - 1.0) * (E - 0.5 * r * (u * u + v * v))
    raise ValueError(f"unknown flow variable {var!r}; one of {VARS}")


def domain_grid(head: dict, blocks, var: str):
    """The frame's variable on the domain's cell grid [ny][nx] (x fastest, row 0 at the bottom),
    NaN where no block lies; returns (grid, dx, dy).  The blocks must share one cell size, as the
    reference's pivot onto a single grid assumes."""
    if "blocks" not in head:
        raise ValueError("frame images are for Cartesian frames (the reference plots those only)")
    bs = head["blocks"]
    dx = (bs[0]["x_right"] - bs[0]["x_left"]) / bs[0]["nx"]
    dy = (bs[0]["y_top"] - bs[0]["y_bottom"]) / bs[0]["ny"]
    for b in bs:
        bdx = (b["x_right"] - b["x_left"]) / b["nx"]
        bdy = (b["y_top"] - b["y_bottom"]) / b["ny"]
        if abs(bdx - dx) > 1e-9 * dx or abs(bdy - dy) > 1e-9 * dy:
            raise ValueError("frame images need one cell size for every block")
    d = head["domain"]
    nx = int(round((d["x_right"] - d["x_left"]) / dx))
    ny = int(round((d["y_top"] - d["y_bottom"]) / dy))
    grid = np.full((ny, nx), np.nan)
    for b, U in zip(bs, blocks):
        i0 = int(round((b["x_left"] - d["x_left"]) / dx))
        j0 = int(round((b["y_bottom"] - d["y_bottom"]) / dy))
        grid[j0:j0 + b["ny"], i0:i0 + b["nx"]] = cell_field(U, var, head["gamma"])
    return grid, dx, dy


def render_grid(grid: np.ndarray, dx: float, dy: float, schlieren: bool, limits=None,
                beta: float = SCHLIEREN_BETA, lam: float = SCHLIEREN_LAMBDA):
    """(imaged field [ny][nx] float64, grey image [ny][nx] uint8), formed on the GPU."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("frame images are formed on the GPU; no CUDA device is visible")
    ny, nx = grid.shape
    f = torch.from_numpy(np.ascontiguousarray(grid, dtype=np.float64)).cuda()
    out = torch.empty_like(f)
    img = torch.empty((ny, nx), dtype=torch.uint8, device="cuda")
    lim = (C.c_double * 2)(*limits) if limits is not None else None
    stream = torch.cuda.current_stream().cuda_stream
    check(lib().hf_render_gray(f.data_ptr(), nx, ny, dx, dy, int(schlieren), beta, lam, lim,
                               out.data_ptr(), img.data_ptr(), stream))
    torch.cuda.synchronize()
    return out.cpu().numpy(), img.cpu().numpy()


def write_png(path: str, img: np.ndarray) -> None:
    """8-bit greyscale PNG (row 0 of img at the top of the picture)."""
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape
    raw = b"".join(b"\x00" + img[r].tobytes() for r in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n")
        fh.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 0, 0, 0, 0)))
        fh.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        fh.write(chunk(b"IEND", b""))


def read_png(path: str) -> np.ndarray:
    """Reads back what write_png wrote (8-bit grey, filter 0 rows)."""
    with open(path, "rb") as fh:
        data = fh.read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    w = h = 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[r * (w + 1) + 1:(r + 1) * (w + 1)] for r in range(h)]
    return np.frombuffer(b"".join(rows), np.uint8).reshape(h, w)


def render_frame(frame_path: str, png_path: str, var: str = "rho", limits=None) -> np.ndarray:
    """One frame file to one PNG; var is a flow variable or "<variable>-gradient"."""
    head, blocks = fr.read_frame(frame_path)
    schlieren = var.endswith("-gradient")
    grid, dx, dy = domain_grid(head, blocks, var.replace("-gradient", ""))
    _, img = render_grid(grid, dx, dy, schlieren, limits)
    write_png(png_path, img[::-1])      # y up, as imshow(origin='lower')
    return img


def render_frames(frames_dir: str, out_dir: str, var: str = "rho", limits=None) -> list[str]:
    """Every results_*.hfb frame of a run, in order, to out_dir/frame_%06d.png."""
    os.makedirs(out_dir, exist_ok=True)
    paths = []
    for k, f in enumerate(sorted(glob.glob(os.path.join(frames_dir, "results_*.hfb")))):
        p = os.path.join(out_dir, "frame_%06d.png" % k)
        render_frame(f, p, var, limits)
        paths.append(p)
    return paths


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("frames_dir")
    ap.add_argument("out_dir")
    ap.add_argument("--var", default="rho", help="rho, u, v, p (or rho_u, rho_v, E), or '<var>-gradient'")
    ap.add_argument("--limits", default=None, help="'lo,hi' range of the grey scale (default: data range)")
    a = ap.parse_args(argv)
    limits = tuple(float(x) for x in a.limits.split(",")) if a.limits else None
    for p in render_frames(a.frames_dir, a.out_dir, a.var, limits):
        print(p)


if __name__ == "__main__":
    main()
