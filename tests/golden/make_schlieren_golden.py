"""Generates tests/golden/render_schlieren.npz by running the reference's own schlieren method,
EulerBlockStructuredVisualisation2D._normalised_gradient_exponential_schlieren
(src/visualisation/euler/euler_2d.py:214-295), on seeded fields.  The module's plotting and CLI
imports (matplotlib, pandas, click) are not installed here and the method does not use them, so
stand-in modules satisfy those imports.  Run where the reference tree exists:

    python tests/golden/make_schlieren_golden.py
"""
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import reference_root  # noqa: E402

REF = os.path.join(reference_root(), "src", "visualisation", "euler", "euler_2d.py")


def load_reference():
    for name in ("matplotlib", "matplotlib.pyplot", "pandas"):
        sys.modules.setdefault(name, types.ModuleType(name))
    click = types.ModuleType("click")
    click.command = lambda *a, **k: (lambda f: f)
    click.option = lambda *a, **k: (lambda f: f)
    sys.modules.setdefault("click", click)
    spec = importlib.util.spec_from_file_location("ref_euler_2d", REF)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def field(nx, ny, seed, hole):
    """A shock-like front, a smooth wave and noise on [0,1] x [0, ny/nx]; NaN in `hole` cells
    (a region no block covers, as the forward-facing step's corner)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / nx
    X, Y = np.meshgrid(x, y, indexing="ij")
    f = 1.0 + 0.8 * np.tanh((X - 0.3 - 0.2 * Y) / 0.01) + 0.2 * np.sin(9 * X) * np.cos(7 * Y)
    f += 1e-3 * rng.standard_normal(f.shape)
    if hole:
        f[int(0.6 * nx):, : int(0.2 * ny)] = np.nan
    return f


def main():
    mod = load_reference()
    out = {}
    for k, (nx, ny, seed, hole) in enumerate([(64, 48, 1, False), (120, 40, 2, True), (7, 5, 3, False)]):
        vis = object.__new__(mod.EulerBlockStructuredVisualisation2D)
        vis.extents = [0.0, 1.0, 0.0, ny / nx]
        vis.cells = (nx, ny)
        f = field(nx, ny, seed, hole)
        out[f"in{k}"] = f
        out[f"out{k}"] = vis._normalised_gradient_exponential_schlieren(f.copy())
        out[f"dx{k}"] = (vis.extents[1] - vis.extents[0]) / vis.cells[0]
        out[f"dy{k}"] = (vis.extents[3] - vis.extents[2]) / vis.cells[1]
    out["source"] = np.array("euler_2d.py:214-295 run on seeded fields (x-major, NaN = no block)")
    np.savez_compressed(os.path.join(HERE, "render_schlieren.npz"), **out)
    print("wrote render_schlieren.npz")


if __name__ == "__main__":
    main()
