"""Triangular mesh generator and the extended HyperFlow mesh text format.

The reference's unstructured solver reads quadrilateral meshes written by
src/mesh_generation/generate_block_mesh.py (format written at 217-246):

    CELLS
    <cell count>
    x1 y1 x2 y2 x3 y3 x4 y4          one line per cell, vertices in order
    EDGES
    <edge count>
    <int>                            one line per (cell, edge) pair, cell by cell

where the int is the boundary code used when the edge has no neighbour
(src/fvm_2d_uns/scheme/boundary/boundary.h:12: -1 Reflective, -2 Transmissive,
-3 Inlet).  The same format carries triangles here: a cell line with 6 numbers is a
triangle.  Coordinates are written with repr(), so they read back bit-exactly.

The binary format holds the same content in a fixed little-endian layout that loads without
number parsing (``hmshb_bytes``; the loader tells the two apart by its magic):

    bytes 0..7    b"HFMESHB1"
    bytes 8..15   cell count, int64
    bytes 16..23  pair count (the cells' vertex counts summed), int64
    int32 x cells vertices per cell (3 or 4)
    int32 x pairs boundary code per (cell, edge) pair, in the EDGES order
    zero padding to a multiple of 8 bytes
    float64 x 2 x pairs  the cells' vertices (x, y), in order

``jittered_hole_mesh`` builds the circular-hole channel of the 1M-cell workload: a
seeded jittered lattice (jitter 0.3 h) over [0,4]x[0,2], points on the circle of radius
0.25 at (1,1), Delaunay triangulation, triangles inside the hole removed, every triangle
counter-clockwise, and cells in Morton (Z-curve) order of their centroids so neighbours
sit close in memory.  The output is canonical (sorted), so every machine gets the same
mesh from the same arguments.
"""
from __future__ import annotations

import math

import numpy as np

REFLECTIVE, TRANSMISSIVE, INLET = -1, -2, -3


def _morton(ix: np.ndarray, iy: np.ndarray) -> np.ndarray:
    def spread(v):
        v = v.astype(np.uint64) & np.uint64(0xFFFFFFFF)
        v = (v | (v << np.uint64(16))) & np.uint64(0x0000FFFF0000FFFF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF00FF00FF)
        v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F0F0F0F0F)
        v = (v | (v << np.uint64(2))) & np.uint64(0x3333333333333333)
        v = (v | (v << np.uint64(1))) & np.uint64(0x5555555555555555)
        return v
    return spread(ix) | (spread(iy) << np.uint64(1))


def jittered_hole_mesh(target_cells: int = 1_000_000, seed: int = 0, x0=0.0, x1=4.0, y0=0.0,
                       y1=2.0, hole=(1.0, 1.0, 0.25), jitter=0.3):
    """Returns (verts [ncells,3,2] float64, edge_codes [ncells,3] int32).

    edge_codes[c, k] is the boundary code of edge k (vertex k -> k+1) of cell c when
    that edge lies on the domain boundary, else 0 (interior edges are matched to their
    neighbour by the loader)."""
    from scipy.spatial import Delaunay

    cx, cy, r = hole
    area = (x1 - x0) * (y1 - y0) - math.pi * r * r
    h = math.sqrt(area / (target_cells / 2.0))       # ~2 triangles per lattice point
    nx = int(round((x1 - x0) / h))
    ny = int(round((y1 - y0) / h))
    hx, hy = (x1 - x0) / nx, (y1 - y0) / ny
    rng = np.random.default_rng(seed)
    gi, gj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    gi, gj = gi.ravel(), gj.ravel()
    px = x0 + gi * hx
    py = y0 + gj * hy
    interior = (gi > 0) & (gi < nx) & (gj > 0) & (gj < ny)
    jx = rng.uniform(-jitter, jitter, px.shape) * hx
    jy = rng.uniform(-jitter, jitter, py.shape) * hy
    px = np.where(interior, px + jx, px)
    py = np.where(interior, py + jy, py)
    # boundary points slide along their own side only
    on_x = ((gj == 0) | (gj == ny)) & (gi > 0) & (gi < nx)
    on_y = ((gi == 0) | (gi == nx)) & (gj > 0) & (gj < ny)
    px = np.where(on_x, px + jx, px)
    py = np.where(on_y, py + jy, py)
    keep = (px - cx) ** 2 + (py - cy) ** 2 > (r + 0.5 * h) ** 2
    px, py = px[keep], py[keep]
    nc = int(math.ceil(2 * math.pi * r / h))
    th = np.arange(nc) * (2 * math.pi / nc)
    px = np.concatenate([px, cx + r * np.cos(th)])
    py = np.concatenate([py, cy + r * np.sin(th)])
    pts = np.stack([px, py], 1)
    tri = Delaunay(pts).simplices.astype(np.int64)
    P = pts[tri]                                          # [T,3,2]
    cen = P.mean(1)
    tri = tri[(cen[:, 0] - cx) ** 2 + (cen[:, 1] - cy) ** 2 > r * r]
    # counter-clockwise, smallest vertex index first (canonical)
    P = pts[tri]
    cross = (P[:, 1, 0] - P[:, 0, 0]) * (P[:, 2, 1] - P[:, 0, 1]) - \
            (P[:, 1, 1] - P[:, 0, 1]) * (P[:, 2, 0] - P[:, 0, 0])
    tri = np.where((cross < 0)[:, None], tri[:, [0, 2, 1]], tri)
    rot = np.argmin(tri, 1)
    tri = np.stack([tri[np.arange(len(tri)), (rot + k) % 3] for k in range(3)], 1)
    # Morton order of centroids, ties by vertex indices
    cen = pts[tri].mean(1)
    q = 1 << 20
    ix = np.clip(((cen[:, 0] - x0) / (x1 - x0) * q).astype(np.int64), 0, q - 1)
    iy = np.clip(((cen[:, 1] - y0) / (y1 - y0) * q).astype(np.int64), 0, q - 1)
    order = np.lexsort((tri[:, 2], tri[:, 1], tri[:, 0], _morton(ix, iy)))
    tri = tri[order]
    verts = pts[tri]
    # boundary codes: edges used by one triangle only
    e = np.stack([tri, np.roll(tri, -1, 1)], 2).reshape(-1, 2)     # (c,k) -> (a,b)
    key = np.minimum(e[:, 0], e[:, 1]) * (len(pts) + 1) + np.maximum(e[:, 0], e[:, 1])
    _, inv, cnt = np.unique(key, return_inverse=True, return_counts=True)
    boundary = cnt[inv] == 1
    a, b = pts[e[:, 0]], pts[e[:, 1]]
    mid = 0.5 * (a + b)
    codes = np.zeros(len(e), dtype=np.int32)
    on_hole = np.abs(np.hypot(mid[:, 0] - cx, mid[:, 1] - cy) - r) < 0.25 * h
    on_left = np.abs(mid[:, 0] - x0) < 1e-9
    codes[boundary] = TRANSMISSIVE
    codes[boundary & on_left] = INLET
    codes[boundary & on_hole] = REFLECTIVE
    return verts, codes.reshape(-1, 3)


def write_hmsh(path: str, verts, codes) -> None:
    """Writes cells (3 or 4 vertices each) and per-edge codes in the reference's format."""
    with open(path, "w") as f:
        f.write("CELLS\n%d\n" % len(verts))
        for cell in verts:
            f.write(" ".join("%r %r" % (float(x), float(y)) for x, y in cell) + "\n")
        n = sum(len(c) for c in codes)
        f.write("EDGES\n%d\n" % n)
        for row in codes:
            for c in row:
                f.write("%d\n" % int(c))


def hmsh_text(verts, codes) -> str:
    lines = ["CELLS", str(len(verts))]
    lines += [" ".join("%r %r" % (float(x), float(y)) for x, y in cell) for cell in verts]
    lines += ["EDGES", str(sum(len(c) for c in codes))]
    lines += [str(int(c)) for row in codes for c in row]
    return "\n".join(lines) + "\n"


MESHB_MAGIC = b"HFMESHB1"


def hmshb_bytes(verts, codes) -> bytes:
    """The binary mesh format of cells (3 or 4 vertices each) and their per-edge codes."""
    nv = np.array([len(c) for c in verts], dtype="<i4")
    flat_codes = np.array([int(c) for row in codes for c in row], dtype="<i4")
    xy = np.array([float(z) for cell in verts for pt in cell for z in pt], dtype="<f8")
    if len(flat_codes) != int(nv.sum()) or len(xy) != 2 * int(nv.sum()):
        raise ValueError("one code and one vertex per (cell, edge) pair")
    head = MESHB_MAGIC + np.array([len(nv), int(nv.sum())], dtype="<i8").tobytes()
    ints = nv.tobytes() + flat_codes.tobytes()
    pad = b"\0" * ((-(len(head) + len(ints))) % 8)
    return head + ints + pad + xy.tobytes()


def write_hmshb(path: str, verts, codes) -> None:
    with open(path, "wb") as f:
        f.write(hmshb_bytes(verts, codes))


def read_hmshb(data: bytes):
    """(verts, codes) from the binary format: per cell a list of (x, y) and a list of codes."""
    if data[:8] != MESHB_MAGIC:
        raise ValueError("not a binary mesh")
    n, npairs = (int(x) for x in np.frombuffer(data, "<i8", 2, 8))
    nv = np.frombuffer(data, "<i4", n, 24)
    codes = np.frombuffer(data, "<i4", npairs, 24 + 4 * n)
    off = 24 + 4 * (n + npairs)
    off += (-off) % 8
    xy = np.frombuffer(data, "<f8", 2 * npairs, off).reshape(-1, 2)
    if off + 16 * npairs != len(data) or int(nv.sum()) != npairs:
        raise ValueError("binary mesh: size does not match the counts")
    starts = np.concatenate([[0], np.cumsum(nv)])
    verts = [[tuple(p) for p in xy[starts[c]:starts[c + 1]].tolist()] for c in range(n)]
    return verts, [codes[starts[c]:starts[c + 1]].tolist() for c in range(n)]


def read_hmsh(text: str):
    """(verts, codes) from the text format."""
    lines = text.split("\n")
    if not lines[0].startswith("CELLS"):
        raise ValueError("expected CELLS header")
    n = int(lines[1])
    verts = []
    for line in lines[2:2 + n]:
        z = [float(t) for t in line.split()]
        verts.append([(z[2 * k], z[2 * k + 1]) for k in range(len(z) // 2)])
    if not lines[2 + n].startswith("EDGES"):
        raise ValueError("expected EDGES header")
    flat = [int(t) for t in lines[4 + n:] if t.strip()]
    codes, k = [], 0
    for cell in verts:
        codes.append(flat[k:k + len(cell)])
        k += len(cell)
    return verts, codes


def channel_case(mesh_file: str, cfl: float = 0.5, inflow=(1.4, 2.0, 0.0, 1.0),
                 t_end: float = 1.0e9) -> dict:
    """Case file of the reference's unstructured solver (parser keys of
    src/fvm_2d_uns/simulation/parser/parser.cpp) for a Mach 2 inflow channel."""
    return {
        "model": {"model": "EulerIdealGas", "gamma": 1.4},
        "mesh": {"type": "hyperflow_unstructured", "file": mesh_file,
                 "boundaries": {"inlet": list(inflow)}},
        "domain": {"x_left": 0.0, "x_right": 4.0, "y_bottom": 0.0, "y_top": 2.0,
                   "boundaries": [[[0.0, 0.0], [4.0, 0.0], [4.0, 2.0], [0.0, 2.0]]]},
        "initial_condition": {"type": "Constant", "variables": "Primitive", "init_state": list(inflow)},
        "scheme": {"type": "Godunov", "riemann": "HLLCEuler", "ode": "ForwardEuler"},
        "simulation": {"cfl": cfl, "t_start": 0.0, "t_end": t_end,
                       "animation": {"duration": 1.0, "fps": 1.0}},
    }
