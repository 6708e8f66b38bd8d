"""Test infrastructure only: the exact solution of the 1D Riemann problem for the ideal-gas
Euler equations, for known-answer checks of the solvers (the reference ships its Toro test 1
case, cases/fvm_2d_cart/shock_tubes/toro/toro_shock_tube_01_*.json, without any check).

Written from the mathematics of E. F. Toro, "Riemann Solvers and Numerical Methods for Fluid
Dynamics" (3rd ed., 2009), chapter 4: the star-region pressure p* is the root of
f(p) = f_L(p) + f_R(p) + (u_R - u_L), where f_K is the shock (Rankine-Hugoniot) branch for
p > p_K and the rarefaction (isentropic) branch otherwise; it is found by Newton's method from
the primitive-variable estimate.  u* = (u_L + u_R)/2 + (f_R(p*) - f_L(p*))/2.  The solution is
self-similar in S = (x - x0)/t and is sampled wave by wave (section 4.5): left of the contact
the left shock or rarefaction fan, right of it the right one.
"""
from __future__ import annotations

import math

import numpy as np


def _fk(p: float, rho: float, pk: float, ck: float, g: float):
    """f_K(p) and its derivative."""
    if p > pk:   # shock
        A = 2.0 / ((g + 1.0) * rho)
        B = (g - 1.0) / (g + 1.0) * pk
        q = math.sqrt(A / (p + B))
        return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (p + B))
    r = p / pk   # rarefaction
    return (2.0 * ck / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0),
            r ** (-(g + 1.0) / (2.0 * g)) / (rho * ck))


def star_state(WL, WR, g: float = 1.4):
    """(p*, u*) of the Riemann problem between primitive states W = (rho, u, p)."""
    rl, ul, pl = (float(x) for x in WL)
    rr, ur, pr = (float(x) for x in WR)
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    if 2.0 * (cl + cr) / (g - 1.0) <= ur - ul:
        raise ValueError("the initial states generate a vacuum")
    p = max(1e-10, 0.5 * (pl + pr) - 0.125 * (ur - ul) * (rl + rr) * (cl + cr))
    for _ in range(200):
        fl, dl = _fk(p, rl, pl, cl, g)
        fr, dr = _fk(p, rr, pr, cr, g)
        pn = max(1e-14, p - (fl + fr + ur - ul) / (dl + dr))
        done = abs(pn - p) <= 1e-15 * 0.5 * (pn + p)
        p = pn
        if done:
            break
    fl, _ = _fk(p, rl, pl, cl, g)
    fr, _ = _fk(p, rr, pr, cr, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(WL, WR, S: np.ndarray, g: float = 1.4) -> np.ndarray:
    """Primitive states [3][len(S)] (rho, u, p) at the similarity coordinates S = (x - x0)/t."""
    rl, ul, pl = (float(x) for x in WL)
    rr, ur, pr = (float(x) for x in WR)
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    ps, us = star_state(WL, WR, g)
    gm, gp = (g - 1.0) / (g + 1.0), (g + 1.0) / (2.0 * g)
    out = np.empty((3, len(S)))
    for k, s in enumerate(np.asarray(S, dtype=float)):
        if s <= us:   # left of the contact
            if ps > pl:   # left shock
                sl = ul - cl * math.sqrt(gp * ps / pl + (g - 1.0) / (2.0 * g))
                w = (rl, ul, pl) if s <= sl else (rl * (ps / pl + gm) / (gm * ps / pl + 1.0), us, ps)
            else:         # left rarefaction
                shl, stl = ul - cl, us - cl * (ps / pl) ** ((g - 1.0) / (2.0 * g))
                if s <= shl:
                    w = (rl, ul, pl)
                elif s > stl:
                    w = (rl * (ps / pl) ** (1.0 / g), us, ps)
                else:
                    c = 2.0 / (g + 1.0) * (cl + 0.5 * (g - 1.0) * (ul - s))
                    w = (rl * (c / cl) ** (2.0 / (g - 1.0)), 2.0 / (g + 1.0) * (cl + 0.5 * (g - 1.0) * ul + s),
                         pl * (c / cl) ** (2.0 * g / (g - 1.0)))
        else:            # right of the contact
            if ps > pr:   # right shock
                sr = ur + cr * math.sqrt(gp * ps / pr + (g - 1.0) / (2.0 * g))
                w = (rr, ur, pr) if s >= sr else (rr * (ps / pr + gm) / (gm * ps / pr + 1.0), us, ps)
            else:         # right rarefaction
                shr, str_ = ur + cr, us + cr * (ps / pr) ** ((g - 1.0) / (2.0 * g))
                if s >= shr:
                    w = (rr, ur, pr)
                elif s <= str_:
                    w = (rr * (ps / pr) ** (1.0 / g), us, ps)
                else:
                    c = 2.0 / (g + 1.0) * (cr - 0.5 * (g - 1.0) * (ur - s))
                    w = (rr * (c / cr) ** (2.0 / (g - 1.0)), 2.0 / (g + 1.0) * (-cr + 0.5 * (g - 1.0) * ur + s),
                         pr * (c / cr) ** (2.0 * g / (g - 1.0)))
        out[:, k] = w
    return out


def cell_averages(WL, WR, x0: float, t: float, edges: np.ndarray, g: float = 1.4, sub: int = 16) -> np.ndarray:
    """Cell averages [3][ncells] (rho, u, p) of the exact solution over the cells between
    consecutive edges, by the midpoint rule on sub points per cell."""
    edges = np.asarray(edges, dtype=float)
    f = (np.arange(sub) + 0.5) / sub
    x = (edges[:-1, None] + (edges[1:] - edges[:-1])[:, None] * f[None, :]).ravel()
    W = sample(WL, WR, (x - x0) / t, g)
    return W.reshape(3, len(edges) - 1, sub).mean(axis=2)
