"""Oracle (test infrastructure only) for the frame images: a numpy restatement of the
reference's "schlieren-like" normalised exponentiated gradient,
EulerBlockStructuredVisualisation2D._normalised_gradient_exponential_schlieren
(src/visualisation/euler/euler_2d.py:214-295), pinned against fixtures generated by running
that method itself (tests/golden/make_schlieren_golden.py), and the linear grey map the GPU image
kernel applies.  Layout as the reference's: f[x][y]."""
from __future__ import annotations

import numpy as np

BETA = 1.0      # euler_2d.py:185-186
LAMBDA = 15.0


def schlieren(f: np.ndarray, dx: float, dy: float, beta: float = BETA, lam: float = LAMBDA) -> np.ndarray:
    """euler_2d.py:245-295: central differences over interior cells (the loops skip the
    boundary rows and columns, whose gradient stays 0), the maximum over interior cells whose
    gradient is a number, then beta * exp(-lambda * g / max) everywhere."""
    with np.errstate(invalid="ignore", divide="ignore"):
        g = np.zeros(f.shape)
        divx = (f[2:, 1:-1] - f[:-2, 1:-1]) / (2.0 * dx)
        divy = (f[1:-1, 2:] - f[1:-1, :-2]) / (2.0 * dy)
        g[1:-1, 1:-1] = np.sqrt(divx * divx + divy * divy)
        inner = g[1:-1, 1:-1]
        mx = np.nanmax(inner) if not np.isnan(inner).all() else -1e6   # the reference's start value
        return beta * np.exp(-lam * g / mx)


def grey(v: np.ndarray, limits=None) -> np.ndarray:
    """The image kernel's map: limits (or the finite range) onto 0..255, rounded half up; NaN 0."""
    fin = v[np.isfinite(v)]
    lo, hi = limits if limits is not None else ((fin.min(), fin.max()) if fin.size else (0.0, 1.0))
    span = hi - lo if hi > lo else 1.0
    with np.errstate(invalid="ignore"):
        t = np.clip((v - lo) / span, 0.0, 1.0)
        out = np.floor(255.0 * t + 0.5)
    out[np.isnan(v)] = 0
    return out.astype(np.uint8)
