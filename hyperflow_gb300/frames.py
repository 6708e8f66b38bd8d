"""Frame files: full-precision binary frames, and the reference's CSV text from them.

The reference writes one CSV per frame (EulerIdealGasDataOutput::to_file,
src/fvm_2d_cart/simulation/output/euler_data_output/euler_data_output.cpp:37-84) with the
stream's default 6 significant digits.  The GPU path captures frames on the device at the
same points (``CartSolver.solve(out_dir=...)``) and stores them here as binary files:

    bytes 0..7    b"HFFRAME1"
    bytes 8..15   header length H, little-endian uint64
    H bytes       JSON header: index, t, t_start, t_end, gamma, domain extents, and per block
                  nx, ny and its extents
    zero padding  to the next multiple of 64 bytes
    data          float64 little-endian; per block, in order, the interior cells SoA
                  [var][y][x] (x fastest), vars rho, rho*u, rho*v, E

``to_csv`` writes the reference's text for a frame -- the same metadata lines, header, row
order (blocks, then x, then y) and cell centroids (MeshBlock::calculate_centroids,
mesh_block.cpp:239-257), with u, v, p from EulerIdealGasModel::cons_to_prim
(euler_ideal_gas.cpp:76-92) -- so tools that read the reference's results_%06d.csv files read
these too.
"""
from __future__ import annotations

import json
import os
import queue
import threading

import numpy as np

MAGIC = b"HFFRAME1"
ALIGN = 64


def case_meta(case: dict) -> dict:
    """Extents and time window of a case, as the frame header records them."""
    dom = case["domain"]
    blocks = []
    for blk in case["mesh"]["blocks"]:
        e = blk["extents"]
        blocks.append({"nx": int(blk["x_cells"]), "ny": int(blk["y_cells"]),
                       "x_left": float(e["x_left"]), "x_right": float(e["x_right"]),
                       "y_bottom": float(e["y_bottom"]), "y_top": float(e["y_top"])})
    sim = case["simulation"]
    return {"gamma": float(case["model"]["gamma"]),
            "ghost": 1 if case["scheme"]["type"] == "Godunov" else 2,
            "t_start": float(sim["t_start"]), "t_end": float(sim["t_end"]),
            "domain": {k: float(dom[k]) for k in ("x_left", "x_right", "y_bottom", "y_top")},
            "blocks": blocks}


def uns_case_meta(case: dict, ncells: int) -> dict:
    """Frame header fields of an unstructured case (the state is one [4][ncells] array)."""
    dom, sim = case["domain"], case["simulation"]
    return {"gamma": float(case["model"]["gamma"]), "ncells": int(ncells),
            "t_start": float(sim["t_start"]), "t_end": float(sim["t_end"]),
            "domain": {k: float(dom[k]) for k in ("x_left", "x_right", "y_bottom", "y_top")}}


def write_frame(path: str, meta: dict, index: int, t: float, blocks) -> None:
    """blocks: per block an array [4][ny][nx] (interior cells); for an unstructured case
    (meta without "blocks") one array [4][ncells]."""
    head = dict(meta, format="hyperflow-gb300 frame", version=1, index=int(index), t=float(t),
                vars=["rho", "rho_u", "rho_v", "E"])
    hj = json.dumps(head).encode()
    pad = (-(len(MAGIC) + 8 + len(hj))) % ALIGN
    with open(path, "wb") as fh:
        fh.write(MAGIC)
        fh.write(np.uint64(len(hj)).tobytes())
        fh.write(hj)
        fh.write(b"\0" * pad)
        for U in blocks:
            np.ascontiguousarray(U, dtype="<f8").tofile(fh)


def read_frame(path: str):
    """Returns (header dict, list of per-block [4][ny][nx] arrays)."""
    with open(path, "rb") as fh:
        raw = fh.read()
    if raw[:8] != MAGIC:
        raise ValueError(f"{path}: not a frame file")
    hl = int(np.frombuffer(raw[8:16], "<u8")[0])
    head = json.loads(raw[16:16 + hl].decode())
    off = 16 + hl
    off += (-off) % ALIGN
    blocks = []
    shapes = [(4, b["ny"], b["nx"]) for b in head["blocks"]] if "blocks" in head else [(4, head["ncells"])]
    for shp in shapes:
        n = int(np.prod(shp))
        blocks.append(np.frombuffer(raw, "<f8", n, off).reshape(shp).copy())
        off += 8 * n
    return head, blocks


def _g(x: float) -> str:
    return "%g" % x


def _csv_head(head: dict):
    d = head["domain"]
    return [f"X_LEFT={_g(d['x_left'])}", f"X_RIGHT={_g(d['x_right'])}",
            f"Y_BOTTOM={_g(d['y_bottom'])}", f"Y_TOP={_g(d['y_top'])}",
            f"T_START={_g(head['t_start'])}", f"T_END={_g(head['t_end'])}", f"T={_g(head['t'])}", "",
            "x,y,rho,rho_u,rho_v,E,u,v,p"]


def _row(x, y, r, ru, rv, E, gm1):
    # EulerIdealGasModel::cons_to_prim, euler_ideal_gas.cpp:76-92
    u = ru / r
    v = rv / r
    p = gm1 * (E - 0.5 * r * (u * u + v * v))
    return ",".join(_g(z) for z in (x, y, r, ru, rv, E, u, v, p))


def uns_csv_text(head: dict, U, centroids) -> str:
    """The reference's unstructured CSV text of one frame (src/fvm_2d_uns/simulation/output/
    euler_data_output/euler_data_output.cpp:37-82): cells in mesh order, centroid first."""
    out = _csv_head(head)
    gm1 = head["gamma"] - 1.0
    for c in range(U.shape[1]):
        out.append(_row(float(centroids[0, c]), float(centroids[1, c]), float(U[0, c]), float(U[1, c]),
                        float(U[2, c]), float(U[3, c]), gm1))
    return "\n".join(out) + "\n"


def csv_text(head: dict, blocks) -> str:
    """The reference's CSV text of one frame (euler_data_output.cpp:48-82)."""
    out = _csv_head(head)
    g = head["ghost"]
    gm1 = head["gamma"] - 1.0
    for b, U in zip(head["blocks"], blocks):
        nx, ny = b["nx"], b["ny"]
        dx = (b["x_right"] - b["x_left"]) / nx
        dy = (b["y_top"] - b["y_bottom"]) / ny
        sx = b["x_left"] - (float(g) - 0.5) * dx
        sy = b["y_bottom"] - (float(g) - 0.5) * dy
        for i in range(nx):
            x = sx + float(i + g) * dx
            for j in range(ny):
                y = sy + float(j + g) * dy
                out.append(_row(x, y, *(float(U[k, j, i]) for k in range(4)), gm1))
    return "\n".join(out) + "\n"


def to_csv(frame_path: str, csv_path: str) -> None:
    head, blocks = read_frame(frame_path)
    with open(csv_path, "w") as fh:
        fh.write(csv_text(head, blocks))


class FrameWriter:
    """Writes frames from a background thread so file output overlaps the device loop.
    fmt "hfb" writes results_%06d.hfb; "csv" writes the reference's results_%06d.csv."""

    def __init__(self, out_dir: str, meta: dict, fmt: str = "hfb", centroids=None):
        if fmt not in ("hfb", "csv"):
            raise ValueError("fmt must be 'hfb' or 'csv'")
        os.makedirs(out_dir, exist_ok=True)
        self.out_dir, self.meta, self.fmt, self.centroids = out_dir, meta, fmt, centroids
        self.paths: list[str] = []
        self._q: queue.Queue = queue.Queue(maxsize=4)
        self._err: BaseException | None = None
        self._t = threading.Thread(target=self._loop, daemon=True)
        self._t.start()

    def _loop(self):
        while True:
            item = self._q.get()
            if item is None:
                return
            index, t, blocks = item
            try:
                path = os.path.join(self.out_dir, f"results_{index:06d}.{self.fmt}")
                if self.fmt == "hfb":
                    write_frame(path, self.meta, index, t, blocks)
                else:
                    head = dict(self.meta, index=index, t=t)
                    text = csv_text(head, blocks) if "blocks" in head else \
                        uns_csv_text(head, blocks[0], self.centroids)
                    with open(path, "w") as fh:
                        fh.write(text)
                self.paths.append(path)
            except BaseException as e:  # reported by close()
                self._err = e

    def put(self, index: int, t: float, blocks) -> None:
        if self._err is not None:
            raise self._err
        self._q.put((index, t, blocks))

    def close(self) -> list[str]:
        self._q.put(None)
        self._t.join()
        if self._err is not None:
            raise self._err
        return self.paths
