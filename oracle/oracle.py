"""Test infrastructure only -- Python bindings for the oracle.

``Oracle``      : the C restatement (oracle/hf_oracle.c, built by ``make -C oracle port``)
                  driven from a case dict in the reference's JSON schema.
``RefCart`` /
``RefUns``      : the reference's own solver sources compiled in place
                  (``make -C oracle ref`` -> oracle/_ref/), available only where the
                  reference tree exists.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module.  The product never does.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libhforacle.so")
REF_CART_LIB = os.path.join(HERE, "_ref", "libhfref_cart.so")
REF_UNS_LIB = os.path.join(HERE, "_ref", "libhfref_uns.so")

MAXB = 16
BC_KIND = {"Transmissive": 0, "Reflective": 1, "Dirichlet": 2, "Internal": 3}
SIDES = ("bottom", "right", "top", "left")


class _Mesh(C.Structure):
    _fields_ = [
        ("scheme", C.c_int), ("limiter", C.c_int), ("nblocks", C.c_int), ("ghost", C.c_int),
        ("gamma", C.c_double), ("cfl", C.c_double), ("calls", C.c_int64),
        ("t", C.c_double), ("t_end", C.c_double),
        ("nx", C.c_int * MAXB), ("ny", C.c_int * MAXB),
        ("xl", C.c_double * MAXB), ("xr", C.c_double * MAXB),
        ("yb", C.c_double * MAXB), ("yt", C.c_double * MAXB),
        ("bc_type", (C.c_int * 4) * MAXB), ("bc_block", (C.c_int * 4) * MAXB),
        ("bc_state", ((C.c_double * 4) * 4) * MAXB),
        ("U", C.c_void_p * MAXB), ("nthreads", C.c_int), ("hllc_errors", C.c_int64),
        ("steps", C.c_int64), ("first_bad", C.c_uint64), ("first_nonpos", C.c_uint64),
    ]


def build_port() -> str:
    """Compile the C restatement (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


_port = None


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        lib = C.CDLL(PORT_LIB)
        d, p, i = C.c_double, C.c_void_p, C.c_int
        lib.hfo_time_step.restype = d
        lib.hfo_time_step.argtypes = [p]
        lib.hfo_run.restype = i
        lib.hfo_run.argtypes = [p, i, i, p]
        lib.hfo_advance.argtypes = [p, d]
        lib.hfo_apply_bcs.argtypes = [p]
        lib.hfo_limiter.restype = d
        lib.hfo_limiter.argtypes = [i, d]
        lib.hfo_hllc.restype = i
        lib.hfo_hllc.argtypes = [d, p, p, i, p]
        lib.hfo_cons_to_prim.argtypes = [d, p, p]
        lib.hfo_prim_to_cons.argtypes = [d, p, p]
        lib.hfo_cons_flux.argtypes = [d, p, i, p]
        lib.hfo_init_quadrant.argtypes = [p, i, d, d, p, p, p, p]
        lib.hfo_init_constant.argtypes = [p, i, p]
        lib.hfo_init_double.argtypes = [p, i, d, d, p, p, p]
        lib.hfo_init_sphere.argtypes = [p, i, d, d, d, p, p]
        lib.hfo_init_shock_bubble.argtypes = [p, i, d, d, d, d, p, p, p]
        lib.hfo_solve.restype = C.c_int64
        lib.hfo_solve.argtypes = [p, d, C.c_int64, p, C.c_int64, p, p, C.c_int64, p]
        lib.hfo_uns_geometry.argtypes = [i, p, p, p, p, p, p]
        lib.hfo_uns_solve.restype = C.c_int64
        lib.hfo_uns_solve.argtypes = [d, d, p, i, p, p, p, p, p, p, p, p, d, d, d, p, p, p,
                                      C.c_int64, p, i]
        lib.hfo_uns_run.restype = i
        lib.hfo_uns_run.argtypes = [d, d, p, i, p, p, p, p, p, p, p, p, i, p, i]
        lib.hfo_uns_first_nonpositive.restype = C.c_int64
        lib.hfo_uns_first_nonpositive.argtypes = [d, i, p]
        _port = lib
    return _port


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def prim_to_cons(w, gamma=1.4):
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.zeros(4)
    port_lib().hfo_prim_to_cons(gamma, _ptr(w), _ptr(out))
    return out


def shock_bubble_states(ic, g):
    """Rankine-Hugoniot post-shock state for a shock of Mach M moving into the ambient gas,
    the bubble state and the ambient state, all conservative."""
    import math
    rho1, u1, v1, p1 = (float(x) for x in ic["ambient_state"])
    M = float(ic["mach"])
    c1 = math.sqrt(g * p1 / rho1)
    p2 = p1 * (1.0 + 2.0 * g / (g + 1.0) * (M * M - 1.0))
    rho2 = rho1 * ((g + 1.0) * M * M / ((g - 1.0) * M * M + 2.0))
    u2 = u1 + M * c1 * (1.0 - rho1 / rho2)
    post = prim_to_cons([rho2, u2, v1, p2], g)
    bub = prim_to_cons([float(ic["bubble_density"]), u1, v1, p1], g)
    amb = prim_to_cons([rho1, u1, v1, p1], g)
    return post, bub, amb


class Oracle:
    """The C restatement of the reference's Cartesian step, set up from a case dict
    the way JSONParser does (parser.cpp:13-488)."""

    def __init__(self, case: dict, nthreads: int = 1):
        self.lib = port_lib()
        self.case = case
        m = _Mesh()
        sch = case["scheme"]["type"]
        m.scheme = 0 if sch == "Godunov" else 1
        m.limiter = 0 if case["scheme"].get("limiter", "MinBee") == "MinBee" else 1
        m.ghost = 1 if m.scheme == 0 else 2
        gamma = float(case["model"]["gamma"])
        m.gamma = gamma
        m.cfl = float(case["simulation"]["cfl"])
        m.t = float(case["simulation"]["t_start"])
        m.t_end = float(case["simulation"]["t_end"])
        m.nthreads = nthreads
        m.first_bad = (1 << 64) - 1
        m.first_nonpos = (1 << 64) - 1
        blocks = case["mesh"]["blocks"]
        m.nblocks = len(blocks)
        self.U = []
        for b, blk in enumerate(blocks):
            e = blk["extents"]
            m.nx[b], m.ny[b] = blk["x_cells"], blk["y_cells"]
            m.xl[b], m.xr[b] = e["x_left"], e["x_right"]
            m.yb[b], m.yt[b] = e["y_bottom"], e["y_top"]
            for s, side in enumerate(SIDES):
                bc = blk["boundaries"][side]
                m.bc_type[b][s] = BC_KIND[bc["type"]]
                if bc["type"] == "Internal":
                    m.bc_block[b][s] = int(bc["block"])
                if bc["type"] == "Dirichlet":
                    st = np.array(bc["flow_state"], dtype=np.float64)
                    if bc["variables"] == "Primitive":
                        st = prim_to_cons(st, gamma)
                    for v in range(4):
                        m.bc_state[b][s][v] = st[v]
            tx, ty = blk["x_cells"] + 2 * m.ghost, blk["y_cells"] + 2 * m.ghost
            U = np.zeros((4, ty, tx))
            self.U.append(U)
            m.U[b] = U.ctypes.data
        self.m = m
        self._init_ic()

    def _states(self, ic, keys):
        out = []
        for k in keys:
            st = np.array(ic[k], dtype=np.float64)
            out.append(st)
        return out

    def _init_ic(self):
        ic = self.case["initial_condition"]
        g = self.m.gamma
        typ = ic["type"]
        prim = ic.get("variables") == "Primitive"
        lib = self.lib
        mp = C.byref(self.m)
        for b in range(self.m.nblocks):
            if typ == "Constant":      # always converted (parser.cpp:317)
                s = prim_to_cons(ic["init_state"], g)
                lib.hfo_init_constant(mp, b, _ptr(s))
            elif typ == "QuadRiemannProblem":
                ne, nw, sw, se = self._states(ic, ["init_ne_state", "init_nw_state",
                                                   "init_sw_state", "init_se_state"])
                if prim:
                    ne, nw, sw, se = (prim_to_cons(x, g) for x in (ne, nw, sw, se))
                lib.hfo_init_quadrant(mp, b, float(ic["x_interface"]), float(ic["y_interface"]),
                                      _ptr(ne), _ptr(nw), _ptr(sw), _ptr(se))
            elif typ == "DoubleRiemannProblem":
                l, mid, r = self._states(ic, ["init_left_state", "init_middle_state",
                                              "init_right_state"])
                if prim:
                    l, mid, r = (prim_to_cons(x, g) for x in (l, mid, r))
                lib.hfo_init_double(mp, b, float(ic["x_lm_interface"]), float(ic["x_mr_interface"]),
                                    _ptr(l), _ptr(mid), _ptr(r))
            elif typ == "SphericalRiemannProblem":   # always converted (parser.cpp:421-422)
                si = prim_to_cons(ic["init_sphere_state"], g)
                so = prim_to_cons(ic["init_ext_state"], g)
                lib.hfo_init_sphere(mp, b, float(ic["radius"]), float(ic["x_origin"]),
                                    float(ic["y_origin"]), _ptr(si), _ptr(so))
            elif typ == "ShockBubble":
                post, bub, amb = shock_bubble_states(ic, g)
                lib.hfo_init_shock_bubble(mp, b, float(ic["shock_x"]), float(ic["bubble_x"]),
                                          float(ic["bubble_y"]), float(ic["bubble_radius"]),
                                          _ptr(post), _ptr(bub), _ptr(amb))
            else:
                raise ValueError(f"initial condition {typ!r} not supported")

    # --- the reference's step pieces ---
    def apply_bcs(self):
        self.lib.hfo_apply_bcs(C.byref(self.m))

    def time_step(self) -> float:
        return self.lib.hfo_time_step(C.byref(self.m))

    def advance(self, dt: float):
        self.lib.hfo_advance(C.byref(self.m), dt)

    def run(self, n: int, clamp_t_end: bool = False) -> np.ndarray:
        dts = np.zeros(max(n, 1))
        k = self.lib.hfo_run(C.byref(self.m), n, int(clamp_t_end), _ptr(dts))
        return dts[:k]

    def frame_interval(self) -> float:
        """simulation.cpp:57: t_end / (anim_duration * anim_fps)"""
        sim = self.case["simulation"]
        return float(sim["t_end"]) / (float(sim["animation"]["duration"]) * float(sim["animation"]["fps"]))

    def solve(self, max_steps: int = 10**9, max_frames: int = 64, max_dts: int = 100000):
        """Simulation::solve with frames: returns (applied dts, frame time labels, frames);
        frames[k] is a list of per-block interior states [4][ny][nx]."""
        dims = [(self.m.nx[b], self.m.ny[b]) for b in range(self.m.nblocks)]
        fcells = sum(4 * nx * ny for nx, ny in dims)
        frames = np.zeros((max_frames, fcells))
        ft = np.zeros(max_frames)
        dts = np.zeros(max_dts)
        nf = C.c_int64()
        k = self.lib.hfo_solve(C.byref(self.m), self.frame_interval(), max_steps, _ptr(dts), max_dts,
                               _ptr(frames), _ptr(ft), max_frames, C.byref(nf))
        out = []
        for f in range(min(nf.value, max_frames)):
            o, blocks = 0, []
            for nx, ny in dims:
                blocks.append(frames[f, o:o + 4 * nx * ny].reshape(4, ny, nx))
                o += 4 * nx * ny
            out.append(blocks)
        return dts[:min(k, max_dts)], ft[:min(nf.value, max_frames)], out

    @property
    def t(self) -> float:
        return self.m.t

    @property
    def calls(self) -> int:
        return self.m.calls

    @property
    def hllc_errors(self) -> int:
        return self.m.hllc_errors

    @property
    def first_bad(self):
        """The earliest zero-flux face (step, block, dir, i, j) as the GPU reports it, or None."""
        k = self.m.first_bad
        if k == (1 << 64) - 1:
            return None
        return {"step": k >> 42, "block": (k >> 38) & 0xF, "dir": (k >> 37) & 1,
                "j": (k >> 19) & 0x3FFFF, "i": k & 0x7FFFF}

    @property
    def first_nonpos(self):
        """The earliest interior cell a step left with density or pressure not positive
        (step, block, i, j) as the GPU reports it, or None."""
        k = self.m.first_nonpos
        if k == (1 << 64) - 1:
            return None
        return {"step": k >> 42, "block": (k >> 38) & 0xF, "j": (k >> 19) & 0x3FFFF, "i": k & 0x7FFFF}

    def state(self, b: int = 0) -> np.ndarray:
        return self.U[b].copy()

    def set_state(self, b: int, U: np.ndarray):
        self.U[b][...] = U


# ----------------------------------------------------------------------------------
# the reference itself (oracle/_ref), for pinning the restatement and making fixtures
# ----------------------------------------------------------------------------------

def ref_available() -> bool:
    return os.path.exists(REF_CART_LIB) and os.path.exists(REF_UNS_LIB)


_refc = None


def ref_cart_lib():
    global _refc
    if _refc is None:
        lib = C.CDLL(REF_CART_LIB)
        p, i, d = C.c_void_p, C.c_int, C.c_double
        lib.hfref_cart_create.restype = p
        lib.hfref_cart_create.argtypes = [C.c_char_p]
        lib.hfref_cart_destroy.argtypes = [p]
        for f in ("hfref_cart_num_blocks", "hfref_cart_num_calls", "hfref_cart_num_steps"):
            getattr(lib, f).restype = i
            getattr(lib, f).argtypes = [p]
        lib.hfref_cart_run.restype = i
        lib.hfref_cart_run.argtypes = [p, i, i]
        lib.hfref_cart_block_dims.argtypes = [p, i, p]
        lib.hfref_cart_get_state.argtypes = [p, i, p]
        lib.hfref_cart_set_state.argtypes = [p, i, p]
        lib.hfref_cart_calls.argtypes = [p, p]
        lib.hfref_cart_step_dts.argtypes = [p, p]
        lib.hfref_cart_apply_bcs.argtypes = [p]
        lib.hfref_cart_solve.restype = i
        lib.hfref_cart_solve.argtypes = [p, C.c_char_p]
        lib.hfref_cart_time.restype = d
        lib.hfref_cart_time.argtypes = [p]
        lib.hfref_hllc.argtypes = [d, p, p, i, p]
        lib.hfref_limiter.restype = d
        lib.hfref_limiter.argtypes = [i, d]
        lib.hfref_cons_to_prim.argtypes = [d, p, p]
        lib.hfref_cons_flux.argtypes = [d, p, i, p]
        _refc = lib
    return _refc


class RefCart:
    """The reference's Cartesian solver built from the same case JSON."""

    def __init__(self, case: dict):
        self.lib = ref_cart_lib()
        self.h = C.c_void_p(self.lib.hfref_cart_create(json.dumps(case).encode()))

    def __del__(self):
        try:
            self.lib.hfref_cart_destroy(self.h)
        except Exception:
            pass

    def run(self, n: int, clamp_t_end: bool = False) -> int:
        return self.lib.hfref_cart_run(self.h, n, int(clamp_t_end))

    def apply_bcs(self):
        self.lib.hfref_cart_apply_bcs(self.h)

    def solve(self, outdir: str):
        """The reference's own Simulation::solve; its CSV frames are written into outdir."""
        if self.lib.hfref_cart_solve(self.h, os.fsencode(outdir)) != 0:
            raise OSError(f"cannot run the reference solve in {outdir}")

    def nblocks(self) -> int:
        return self.lib.hfref_cart_num_blocks(self.h)

    def state(self, b: int = 0) -> np.ndarray:
        dims = (C.c_int * 3)()
        self.lib.hfref_cart_block_dims(self.h, b, dims)
        out = np.zeros((4, dims[1], dims[0]))
        self.lib.hfref_cart_get_state(self.h, b, _ptr(out))
        return out

    def set_state(self, b: int, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self.lib.hfref_cart_set_state(self.h, b, _ptr(U))

    def calls(self) -> np.ndarray:
        n = self.lib.hfref_cart_num_calls(self.h)
        out = np.zeros(max(n, 1))
        self.lib.hfref_cart_calls(self.h, _ptr(out))
        return out[:n]

    def step_dts(self) -> np.ndarray:
        n = self.lib.hfref_cart_num_steps(self.h)
        out = np.zeros(max(n, 1))
        self.lib.hfref_cart_step_dts(self.h, _ptr(out))
        return out[:n]

    def time(self) -> float:
        return self.lib.hfref_cart_time(self.h)


_refu = None


def ref_uns_lib():
    global _refu
    if _refu is None:
        lib = C.CDLL(REF_UNS_LIB)
        p, i = C.c_void_p, C.c_int
        lib.hfref_uns_create.restype = p
        lib.hfref_uns_create.argtypes = [C.c_char_p, i, p, p, p]
        lib.hfref_uns_destroy.argtypes = [p]
        lib.hfref_uns_run.restype = i
        lib.hfref_uns_run.argtypes = [p, i]
        lib.hfref_uns_dts.argtypes = [p, p]
        lib.hfref_uns_get_state.argtypes = [p, p]
        lib.hfref_uns_set_state.argtypes = [p, p]
        lib.hfref_uns_geometry.argtypes = [p, p, p, p, p]
        lib.hfref_uns_solve.restype = i
        lib.hfref_uns_solve.argtypes = [p, C.c_char_p]
        lib.hfref_uns_centroids.argtypes = [p, p]
        lib.hfref_uns_create_file.restype = p
        lib.hfref_uns_create_file.argtypes = [C.c_char_p]
        lib.hfref_uns_cell_edge_indices.restype = C.c_long
        lib.hfref_uns_cell_edge_indices.argtypes = [p, p, C.c_long]
        _refu = lib
    return _refu


class RefUns:
    """The reference's unstructured solver over a mesh given as arrays."""

    def __init__(self, case: dict, nverts: np.ndarray, verts: np.ndarray, pair_nbr: np.ndarray):
        self.lib = ref_uns_lib()
        self.nverts = np.ascontiguousarray(nverts, dtype=np.int32)
        self.verts = np.ascontiguousarray(verts, dtype=np.float64)
        self.nbr = np.ascontiguousarray(pair_nbr, dtype=np.int32)
        self.ncells = len(self.nverts)
        self.npairs = int(self.nverts.sum())
        self.h = C.c_void_p(self.lib.hfref_uns_create(json.dumps(case).encode(), self.ncells,
                                                      _ptr(self.nverts), _ptr(self.verts),
                                                      _ptr(self.nbr)))
        self.nsteps = 0

    @classmethod
    def from_file(cls, case: dict, quiet: bool = True):
        """The reference's own loader (JSONParser::generate_mesh -> LoadStructuredMesh, an O(E^2)
        scan over quadrilaterals) on the case's mesh.file.  quiet: its per-cell progress lines,
        printed to stdout, are dropped."""
        self = cls.__new__(cls)
        self.lib = ref_uns_lib()
        raw = json.dumps(case).encode()
        if quiet:
            import sys
            sys.stdout.flush()
            saved = os.dup(1)
            devnull = os.open(os.devnull, os.O_WRONLY)
            os.dup2(devnull, 1)
            try:
                h = self.lib.hfref_uns_create_file(raw)
            finally:
                os.dup2(saved, 1)
                os.close(saved)
                os.close(devnull)
        else:
            h = self.lib.hfref_uns_create_file(raw)
        if not h:
            raise ValueError("the reference loader refused the mesh")
        self.h = C.c_void_p(h)
        cei = self.cell_edge_indices()
        self.npairs = len(cei)
        self.ncells = int(cei[:, 0].max()) + 1 if self.npairs else 0
        self.nverts = np.bincount(cei[:, 0], minlength=self.ncells).astype(np.int32)
        self.nbr = np.ascontiguousarray(cei[:, 1])
        self.nsteps = 0
        return self

    def cell_edge_indices(self) -> np.ndarray:
        """The mesh's cell_edge_indices, [npairs][3] = (cell, neighbour or code, edge index)."""
        n = self.lib.hfref_uns_cell_edge_indices(self.h, None, 0)
        out = np.zeros((n, 3), np.int32)
        self.lib.hfref_uns_cell_edge_indices(self.h, _ptr(out), n)
        return out

    def __del__(self):
        try:
            self.lib.hfref_uns_destroy(self.h)
        except Exception:
            pass

    def run(self, n: int):
        self.lib.hfref_uns_run(self.h, n)
        self.nsteps += n

    def dts(self) -> np.ndarray:
        out = np.zeros(max(self.nsteps, 1))
        self.lib.hfref_uns_dts(self.h, _ptr(out))
        return out[: self.nsteps]

    def state(self) -> np.ndarray:
        out = np.zeros((4, self.ncells))
        self.lib.hfref_uns_get_state(self.h, _ptr(out))
        return out

    def set_state(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self.lib.hfref_uns_set_state(self.h, _ptr(U))

    def solve(self, outdir: str):
        """The reference's own Simulation::solve; its CSV frames are written into outdir."""
        if self.lib.hfref_uns_solve(self.h, os.fsencode(outdir)) != 0:
            raise OSError(f"cannot run the reference solve in {outdir}")

    def centroids(self) -> np.ndarray:
        out = np.zeros((2, self.ncells))
        self.lib.hfref_uns_centroids(self.h, _ptr(out))
        return out

    def geometry(self):
        ang = np.zeros(self.npairs)
        ln = np.zeros(self.npairs)
        area = np.zeros(self.ncells)
        rin = np.zeros(self.ncells)
        self.lib.hfref_uns_geometry(self.h, _ptr(ang), _ptr(ln), _ptr(area), _ptr(rin))
        return ang, ln, area, rin


EDGE_TOL = 1e-12   # Edge's default tolerance, src/fvm_2d_uns/geometry/edge/edge.h:21


def ref_neighbours(verts, codes, tol: float = EDGE_TOL):
    """The neighbour of every (cell, edge) pair by the reference loader's rule
    (src/fvm_2d_uns/mesh/mesh_structured/mesh_structured.cpp:92-114): pair q (edge A -> B of its
    cell) takes the cell of the LAST pair r, in pair order, for which
    Edge::opposite_edges_equal holds (src/fvm_2d_uns/geometry/edge/edge.cpp:59-71):
    fabs(start_r - B) < tol and fabs(end_r - A) < tol in x and in y; with no such r it keeps its
    code.  Candidates come from a k-d tree over the start points (a radius of 4 tol in the max
    norm), every one is decided by the reference's own comparison.  verts: per cell a sequence
    of (x, y) vertices; codes: per cell its codes.  Returns (nbr int32 per pair, unmatched pairs
    whose code is a cell index)."""
    from scipy.spatial import cKDTree
    S = np.array([p for cell in verts for p in cell], dtype=np.float64).reshape(-1, 2)
    nv = np.array([len(cell) for cell in verts])
    starts = np.concatenate([[0], np.cumsum(nv)])
    nxt = np.arange(len(S)) + 1
    nxt[starts[1:] - 1] = starts[:-1]
    cell = np.repeat(np.arange(len(verts)), nv)
    E = S[nxt]
    flat = np.array([k for cc in codes for k in cc], dtype=np.int64)
    finite = np.isfinite(S).all(axis=1)
    idx = np.nonzero(finite)[0]
    tree = cKDTree(S[idx])
    nbr = np.empty(len(S), np.int32)
    unmatched = 0
    qok = np.isfinite(E).all(axis=1)
    cands = tree.query_ball_point(np.where(qok[:, None], E, 0.0), r=4 * tol, p=np.inf)
    for q in range(len(S)):
        best = -1
        if qok[q]:
            for r in sorted((int(idx[j]) for j in cands[q]), reverse=True):
                if (abs(S[r, 0] - E[q, 0]) < tol and abs(S[r, 1] - E[q, 1]) < tol and
                        abs(E[r, 0] - S[q, 0]) < tol and abs(E[r, 1] - S[q, 1]) < tol):
                    best = r
                    break
        if best >= 0:
            nbr[q] = cell[best]
        else:
            nbr[q] = flat[q]
            unmatched += int(flat[q] >= 0)
    return nbr, unmatched


def uns_geometry(nverts: np.ndarray, verts: np.ndarray):
    """Edge angles/lengths and cell areas/incircle radii via the C restatement."""
    nverts = np.ascontiguousarray(nverts, dtype=np.int32)
    verts = np.ascontiguousarray(verts, dtype=np.float64)
    npairs = int(nverts.sum())
    ang, ln = np.zeros(npairs), np.zeros(npairs)
    area, rin = np.zeros(len(nverts)), np.zeros(len(nverts))
    port_lib().hfo_uns_geometry(len(nverts), _ptr(nverts), _ptr(verts), _ptr(ang), _ptr(ln),
                                _ptr(area), _ptr(rin))
    return ang, ln, area, rin


def uns_solve(gamma, cfl, pair_start, pair_nbr, angle, length, area, rin, inlet, U, t_start,
              t_end, interval, max_frames=64, nthreads=1):
    """Simulation::solve of the restated unstructured solver with its frame cadence; U
    ([4][ncells]) ends at t_end.  Returns (steps, TimeStep calls, frame labels, frames)."""
    c = C.c_int64(0)
    N = U.shape[1]
    frames = np.zeros((max_frames, 4, N))
    ft = np.zeros(max_frames)
    nf = C.c_int64()
    t_out = C.c_double()
    ps = np.ascontiguousarray(pair_start, dtype=np.int32)
    pn = np.ascontiguousarray(pair_nbr, dtype=np.int32)
    inlet = np.ascontiguousarray(inlet, dtype=np.float64)
    k = port_lib().hfo_uns_solve(gamma, cfl, C.byref(c), N, _ptr(ps), _ptr(pn), _ptr(angle),
                                 _ptr(length), _ptr(area), _ptr(rin), _ptr(inlet), _ptr(U), t_start,
                                 t_end, interval, C.byref(t_out), _ptr(frames), _ptr(ft), max_frames,
                                 C.byref(nf), nthreads)
    m = min(nf.value, max_frames)
    return k, c.value, ft[:m], frames[:m]


def uns_first_nonpositive(gamma, U):
    """The least cell of U ([4][ncells]) whose density or pressure is not positive, or None."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    k = port_lib().hfo_uns_first_nonpositive(gamma, U.shape[1], _ptr(U))
    return None if k < 0 else int(k)


def uns_run(gamma, cfl, calls, pair_start, pair_nbr, angle, length, area, rin, inlet, U, n,
            nthreads=1):
    """n steps of the restated unstructured Godunov solver; U ([4][ncells]) updated in place."""
    c = C.c_int64(calls)
    dts = np.zeros(max(n, 1))
    ps = np.ascontiguousarray(pair_start, dtype=np.int32)
    pn = np.ascontiguousarray(pair_nbr, dtype=np.int32)
    inlet = np.ascontiguousarray(inlet, dtype=np.float64)
    port_lib().hfo_uns_run(gamma, cfl, C.byref(c), U.shape[1], _ptr(ps), _ptr(pn), _ptr(angle),
                           _ptr(length), _ptr(area), _ptr(rin), _ptr(inlet), _ptr(U), n,
                           _ptr(dts), nthreads)
    return dts[:n], c.value
