"""Case files in the reference's JSON schema for the standard workloads.

The schema is the one src/fvm_2d_cart/simulation/parser/parser.cpp reads
(keys at parser.cpp:13-43, 104-115, 166-245, 262-308, 432-488).  Every function
returns a plain ``dict`` that serialises to a case file the reference executable
would accept unchanged.
"""
from __future__ import annotations

import json
import math

GAMMA = 1.4

# Four-quadrant Riemann problem of the 256x256 Godunov workload, primitive (rho, u, v, p)
QUAD_NE = [1.5, 0.0, 0.0, 1.5]
QUAD_NW = [0.5323, 1.206, 0.0, 0.3]
QUAD_SW = [0.138, 1.206, 1.206, 0.029]
QUAD_SE = [0.5323, 0.0, 1.206, 0.3]


def _bc(kind: str, **kw) -> dict:
    d = {"type": kind}
    d.update(kw)
    return d


def _block(x0, x1, y0, y1, nx, ny, bottom, right, top, left) -> dict:
    return {
        "extents": {"x_left": x0, "x_right": x1, "y_bottom": y0, "y_top": y1},
        "boundaries": {"bottom": bottom, "right": right, "top": top, "left": left},
        "x_cells": nx,
        "y_cells": ny,
    }


def _domain(x0, x1, y0, y1) -> dict:
    return {"x_left": x0, "x_right": x1, "y_bottom": y0, "y_top": y1,
            "boundaries": [[[x0, y0], [x1, y0], [x1, y1], [x0, y1]]]}


def _scheme(scheme: str, limiter: str | None) -> dict:
    s = {"type": scheme, "riemann": "HLLCEuler", "ode": "ForwardEuler"}
    if scheme == "MUSCLHancock":
        s["limiter"] = limiter or "MinBee"
    return s


# CFL of the generated two-dimensional workloads (batched Riemann problems, shock-bubble,
# learned-solver training data).  The reference's dt takes the CFL number per direction
# (min over dx/(|u|+c) and dy/(|v|+c)), and its unsplit MUSCL-Hancock update is stable only
# while the two directional Courant numbers sum to about 1 or less: at CFL 0.8 the
# shock-bubble flow loses positivity after about 70 steps at 256^2 and above, and 5 of 40
# small batched Riemann problems blow up within 500 steps; at 0.4 none do.
CFL_2D = 0.4


def _simulation(cfl: float, t_end: float) -> dict:
    return {"cfl": cfl, "t_start": 0.0, "t_end": t_end,
            "animation": {"duration": 1.0, "fps": 1.0}}


def quadrant_case(n: int = 256, ny: int | None = None, scheme: str = "Godunov",
                  limiter: str | None = None, cfl: float = 0.8, t_end: float = 1.0e9,
                  split=(0.5, 0.5), states=None, bc: str = "Transmissive",
                  extents=(0.0, 1.0, 0.0, 1.0)) -> dict:
    """Single-block four-quadrant Riemann problem (QuadRiemannProblem IC,
    quadrp.cpp:49-64) -- the 256x256 Godunov parity workload by default."""
    ny = n if ny is None else ny
    ne, nw, sw, se = states if states is not None else (QUAD_NE, QUAD_NW, QUAD_SW, QUAD_SE)
    x0, x1, y0, y1 = extents
    b = _bc(bc)
    return {
        "model": {"model": "EulerIdealGas", "gamma": GAMMA},
        "mesh": {"blocks": [_block(x0, x1, y0, y1, n, ny, b, b, b, b)]},
        "domain": _domain(x0, x1, y0, y1),
        "initial_condition": {
            "type": "QuadRiemannProblem", "variables": "Primitive",
            "x_interface": split[0], "y_interface": split[1],
            "init_ne_state": list(ne), "init_nw_state": list(nw),
            "init_sw_state": list(sw), "init_se_state": list(se),
        },
        "scheme": _scheme(scheme, limiter),
        "simulation": _simulation(cfl, t_end),
    }


def forward_facing_step_case(cells_per_unit: int = 1365, limiter: str = "MinBee",
                             cfl: float = 0.8, t_end: float = 4.0,
                             scheme: str = "MUSCLHancock") -> dict:
    """Mach 3 forward-facing step on [0,3]x[0,1], step at x=0.6 of height 0.2,
    three blocks at a uniform spacing dx = dy = 1/cells_per_unit.

    Block 0 = [0,0.6]x[0,0.2] (below the step's left part), block 1 = [0,0.6]x[0.2,1],
    block 2 = [0.6,3]x[0.2,1].  Inflow (1.4, 3, 0, 1) enters on the left as a
    Dirichlet state in primitive variables (dirichlet_boundary.cpp); walls and the
    step faces are Reflective; the right side is Transmissive; blocks are joined
    by Internal boundaries (internal_boundary.cpp).  The initial state is the
    uniform inflow (Constant IC, constant.cpp:34-40).
    """
    h = cells_per_unit
    n06 = int(round(0.6 * h))
    n02 = int(round(0.2 * h))
    n08 = int(round(0.8 * h))
    n24 = int(round(2.4 * h))
    inflow = [1.4, 3.0, 0.0, 1.0]
    dirich = _bc("Dirichlet", variables="Primitive", flow_state=inflow)
    refl = _bc("Reflective")
    trans = _bc("Transmissive")
    # the spacing is the same in every block only when the cell counts divide evenly
    blocks = [
        _block(0.0, 0.6, 0.0, 0.2, n06, n02, refl, refl, _bc("Internal", block=1), dirich),
        _block(0.0, 0.6, 0.2, 1.0, n06, n08, _bc("Internal", block=0), _bc("Internal", block=2),
               refl, dirich),
        _block(0.6, 3.0, 0.2, 1.0, n24, n08, refl, trans, refl, _bc("Internal", block=1)),
    ]
    return {
        "model": {"model": "EulerIdealGas", "gamma": GAMMA},
        "mesh": {"blocks": blocks},
        "domain": _domain(0.0, 3.0, 0.0, 1.0),
        "initial_condition": {"type": "Constant", "variables": "Primitive", "init_state": inflow},
        "scheme": _scheme(scheme, limiter),
        "simulation": _simulation(cfl, t_end),
    }


def shock_bubble_case(n: int = 2048, scheme: str = "MUSCLHancock", limiter: str = "MinBee",
                      cfl: float = CFL_2D, t_end: float = 0.25, mach: float = 1.22,
                      bubble_density: float = 0.138, radius: float = 0.2, bubble=(0.4, 0.5),
                      shock_x: float = 0.12) -> dict:
    """A Mach 1.22 shock moving in +x through still air (rho 1, p 1) onto a circular bubble of
    density 0.138 and radius 0.2, on [0,1]^2 with transmissive sides (new
    initial_condition type "ShockBubble"; post-shock state from Rankine-Hugoniot)."""
    b = _bc("Transmissive")
    return {
        "model": {"model": "EulerIdealGas", "gamma": GAMMA},
        "mesh": {"blocks": [_block(0.0, 1.0, 0.0, 1.0, n, n, b, b, b, b)]},
        "domain": _domain(0.0, 1.0, 0.0, 1.0),
        "initial_condition": {
            "type": "ShockBubble", "variables": "Primitive", "shock_x": shock_x, "mach": mach,
            "bubble_x": bubble[0], "bubble_y": bubble[1], "bubble_radius": radius,
            "bubble_density": bubble_density, "ambient_state": [1.0, 0.0, 0.0, 1.0],
        },
        "scheme": _scheme(scheme, limiter),
        "simulation": _simulation(cfl, t_end),
    }


def random_quadrant_case(n: int, seed: int, limiter: str = "MinBee", cfl: float = CFL_2D,
                         t_end: float | None = None) -> dict:
    """One four-quadrant Riemann problem drawn like the batched workload's cases (split in
    [0.3,0.7]^2, rho in [0.1,2], p in [0.1,10], u, v in [-1,1]); t_end defaults to the time
    the fastest initial wave needs to cross a quarter of the domain."""
    import numpy as np
    rng = np.random.default_rng(seed)
    split = (float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.3, 0.7)))
    states = [[float(rng.uniform(0.1, 2.0)), float(rng.uniform(-1.0, 1.0)),
               float(rng.uniform(-1.0, 1.0)), float(rng.uniform(0.1, 10.0))] for _ in range(4)]
    if t_end is None:
        smax = max(max(abs(u), abs(v)) + math.sqrt(GAMMA * p / r) for r, u, v, p in states)
        t_end = 0.25 / smax
    return quadrant_case(n, scheme="MUSCLHancock", limiter=limiter, cfl=cfl, split=split,
                         states=states, t_end=t_end)


def batch_manifest(count: int = 512, seed: int = 0, side_min: int = 64, side_max: int = 1024,
                   limiter: str = "MinBee", cfl: float = CFL_2D, scheme: str = "MUSCLHancock") -> dict:
    """The batched workload: `count` independent square four-quadrant Riemann problems on
    [0,1]^2, sides log-uniform in [side_min, side_max] (rounded), split point uniform in
    [0.3,0.7]^2, and per quadrant rho ~ U[0.1,2], p ~ U[0.1,10], u, v ~ U[-1,1]
    (primitive), transmissive on every side, MUSCL-Hancock (or Godunov) + HLLC.  Seeded."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(side_min), math.log(side_max)))))
        split = (float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.3, 0.7)))
        states = []
        for _q in range(4):
            states.append([float(rng.uniform(0.1, 2.0)), float(rng.uniform(-1.0, 1.0)),
                           float(rng.uniform(-1.0, 1.0)), float(rng.uniform(0.1, 10.0))])
        out.append(quadrant_case(n, scheme=scheme, limiter=limiter if scheme == "MUSCLHancock" else None,
                                 cfl=cfl, split=split, states=states))
    return {"cases": out}


def to_json(case: dict) -> str:
    return json.dumps(case, indent=1)


def total_cells(case: dict) -> int:
    return sum(b["x_cells"] * b["y_cells"] for b in case["mesh"]["blocks"])


__all__ = ["quadrant_case", "forward_facing_step_case", "shock_bubble_case", "random_quadrant_case",
           "batch_manifest", "to_json", "total_cells",
           "QUAD_NE", "QUAD_NW", "QUAD_SW", "QUAD_SE", "GAMMA", "math"]
