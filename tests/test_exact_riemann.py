"""Known-answer checks against the exact Riemann solution (oracle/exact_riemann.py, written from
Toro's chapter 4): the exact solver against the star states Toro tabulates for his tests 1-4,
and the reference's Toro test 1 case (cases/fvm_2d_cart/shock_tubes/toro/, Godunov and
MUSCL-Hancock Van Leer, modified Sod problem with u_L = 0.75, x0 = 0.3, t = 0.2): L1 density
error of the oracle (CPU) and of the CUDA path (GPU) against the exact cell averages, and its
decrease under grid refinement."""
import copy
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

WL, WR, X0 = (1.0, 0.75, 1.0), (0.125, 0.0, 0.1), 0.3


@pytest.mark.parametrize("wl, wr, p_star, u_star", [
    ((1.0, 0.0, 1.0), (0.125, 0.0, 0.1), 0.30313, 0.92745),                   # Sod
    ((1.0, -2.0, 0.4), (1.0, 2.0, 0.4), 0.00189, 0.0),                        # 123 problem
    ((1.0, 0.0, 1000.0), (1.0, 0.0, 0.01), 460.894, 19.5975),                 # strong left blast
    ((5.99924, 19.5975, 460.894), (5.99242, -6.19633, 46.0950), 1691.64, 8.68975),  # shock collision
])
def test_exact_star_states_match_published_values(wl, wr, p_star, u_star):
    from oracle.exact_riemann import star_state
    p, u = star_state(wl, wr)
    assert abs(p - p_star) <= 6e-6 * max(1.0, p_star) + 5e-6
    assert abs(u - u_star) <= 6e-6 * max(1.0, abs(u_star)) + 5e-6


def test_exact_solution_conserves_mass_momentum_energy():
    """Over [-1, 1.6] no wave reaches the ends by t = 0.2, so the integrals change only by the
    far states' fluxes: d/dt int U dx = F(W_L) - F(W_R)."""
    from oracle.exact_riemann import sample
    g, t, n = 1.4, 0.2, 208000
    x = -1.0 + (np.arange(n) + 0.5) * (2.6 / n)      # midpoint rule on 2.6 / n
    r, u, p = sample(WL, WR, (x - X0) / t, g)
    U = np.array([r, r * u, p / (g - 1.0) + 0.5 * r * u * u]).sum(axis=1) * (2.6 / n)

    def cons(w):
        r, u, p = w
        return np.array([r, r * u, p / (g - 1.0) + 0.5 * r * u * u])

    def flux(w):
        r, u, p = w
        E = p / (g - 1.0) + 0.5 * r * u * u
        return np.array([r * u, r * u * u + p, u * (E + p)])

    U0 = cons(WL) * (X0 + 1.0) + cons(WR) * (1.6 - X0)
    expect = U0 + t * (flux(WL) - flux(WR))
    np.testing.assert_allclose(U, expect, rtol=2e-5)


def _toro_case(scheme, nx):
    d = np.load(os.path.join(GOLDEN, "frames_toro_shock_tube_01_godunov_hllc_100x5.npz"))
    case = json.loads(str(d["case"]))
    c = copy.deepcopy(case)
    c["mesh"]["blocks"][0]["x_cells"] = nx
    if scheme == "MUSCLHancock":
        c["scheme"] = dict(case["scheme"], type="MUSCLHancock", limiter="VanLeer")
    return c


def _l1(rho, nx, t):
    from oracle.exact_riemann import cell_averages
    ex = cell_averages(WL, WR, X0, t, np.linspace(0.0, 1.0, nx + 1))
    return float(np.mean(np.abs(rho - ex[0][None, :])))


def _oracle_l1(scheme, nx):
    from oracle.oracle import Oracle
    o = Oracle(_toro_case(scheme, nx), nthreads=4)
    while o.t < o.m.t_end:
        o.run(1, True)
    g = o.m.ghost
    return _l1(o.state(0)[0, g:-g, g:-g], nx, o.t), o.t


@pytest.mark.parametrize("scheme, bound100", [("Godunov", 0.0160), ("MUSCLHancock", 0.0070)])
def test_oracle_converges_to_the_exact_toro1_solution(scheme, bound100, port_lib):
    e100, t = _oracle_l1(scheme, 100)
    e400, _ = _oracle_l1(scheme, 400)
    assert t == 0.2
    assert e100 < bound100
    assert e100 / e400 > 2.0          # about first order at the shock and the contact


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["Godunov", "MUSCLHancock"])
def test_gpu_toro1_error_equals_oracle_and_converges(scheme, port_lib):
    """The GPU's L1 density error equals the oracle's at 100 and 400 cells (the states are
    bit-identical) and keeps falling to 1600 cells; MUSCL-Hancock is the more accurate."""
    from hyperflow_gb300 import CartSolver
    errs = {}
    for nx in (100, 400, 1600):
        s = CartSolver(_toro_case(scheme, nx))
        s.run(2 * nx + 100, clamp_t_end=True)   # about 1.1 nx steps reach t_end; the rest are no-ops
        t = s.time()[0]
        assert t == 0.2
        g = 1 if scheme == "Godunov" else 2
        rho = s.state(0)[0, g:-g, g:-g]
        errs[nx] = _l1(rho, nx, t)
        if nx <= 400:
            assert errs[nx] == _oracle_l1(scheme, nx)[0]
    assert errs[100] / errs[400] > 2.0 and errs[400] / errs[1600] > 2.0
    if scheme == "MUSCLHancock":
        assert errs[1600] < 0.001
    else:
        assert errs[1600] < 0.0035


def _tri_strip(nx, ny=4, length=1.0, height=0.05):
    """Toro test 1's tube as triangles: an nx x ny grid of squares, each cut along a diagonal
    (alternating), counter-clockwise; ends transmissive, sides reflective."""
    from hyperflow_gb300 import meshgen
    xs, ys = np.linspace(0.0, length, nx + 1), np.linspace(0.0, height, ny + 1)
    verts, codes = [], []
    for i in range(nx):
        for j in range(ny):
            p00, p10 = (xs[i], ys[j]), (xs[i + 1], ys[j])
            p01, p11 = (xs[i], ys[j + 1]), (xs[i + 1], ys[j + 1])
            tris = [(p00, p10, p11), (p00, p11, p01)] if (i + j) % 2 == 0 else [(p00, p10, p01), (p10, p11, p01)]
            for t in tris:
                verts.append(t)
                cc = []
                for k in range(3):
                    a, b = t[k], t[(k + 1) % 3]
                    if a[1] == b[1] and a[1] in (ys[0], ys[-1]):
                        cc.append(meshgen.REFLECTIVE)
                    elif a[0] == b[0] and a[0] in (xs[0], xs[-1]):
                        cc.append(meshgen.TRANSMISSIVE)
                    else:
                        cc.append(0)
                codes.append(cc)
    return np.array(verts), np.array(codes)


def _uns_toro_state(verts):
    from oracle.oracle import prim_to_cons
    cx = verts[:, :, 0].mean(axis=1)
    left = prim_to_cons([WL[0], WL[1], 0.0, WL[2]])
    right = prim_to_cons([WR[0], WR[1], 0.0, WR[2]])
    return np.where(cx[None, :] <= X0, left[:, None], right[:, None]).astype(np.float64)


def _uns_l1(U, verts, t):
    """L1 density error over the strip, cell by cell against the exact solution at the
    centroid x (area-weighted: every triangle of the strip has the same area)."""
    from oracle.exact_riemann import sample
    cx = verts[:, :, 0].mean(axis=1)
    return float(np.mean(np.abs(U[0] - sample(WL, WR, (cx - X0) / t)[0])))


def _uns_case():
    from hyperflow_gb300 import meshgen
    case = meshgen.channel_case("unused.hmsh", cfl=0.5)
    case["simulation"]["t_end"] = 0.2
    return case


def _uns_oracle(nx):
    """The oracle's Godunov run on the strip (ny = nx / 20, right-angled triangles of equal
    area) up to the first step that ends at or past t = 0.2."""
    from hyperflow_gb300 import meshgen
    from oracle import oracle
    verts, codes = _tri_strip(nx, ny=nx // 20)
    nbr = oracle.ref_neighbours(list(verts), list(codes))[0]
    nv = np.full(len(verts), 3, np.int32)
    ang, ln, area, rin = oracle.uns_geometry(nv, verts.reshape(-1))
    ps = np.concatenate([[0], np.cumsum(nv)]).astype(np.int32)
    U = _uns_toro_state(verts)
    t, calls, steps = 0.0, 0, 0
    while t < 0.2:
        dts, calls = oracle.uns_run(1.4, 0.5, calls, ps, nbr, ang, ln, area, rin, np.zeros(4), U, 1)
        t += dts[0]
        steps += 1
    return verts, codes, U, t, steps


def test_uns_oracle_converges_to_the_exact_toro1_solution(port_lib):
    """Toro test 1 through the unstructured Godunov scheme (rotations, edge normals, the
    reflective sides and transmissive ends) on triangles: the L1 density error at the cell
    centroids falls under refinement."""
    e = {}
    for nx in (80, 160, 320):
        verts, _, U, t, _ = _uns_oracle(nx)
        e[nx] = _uns_l1(U, verts, t)
    assert e[80] < 0.03 and e[80] / e[160] > 1.4 and e[160] / e[320] > 1.4, e


@pytest.mark.gpu
def test_uns_gpu_toro1_equals_oracle(port_lib):
    """The CUDA unstructured path (per-pair mode) on the same strip and steps: bit-exact to
    the oracle, so its error against the exact solution is the oracle's."""
    from hyperflow_gb300 import UnsSolver, meshgen
    verts, codes, U, t, steps = _uns_oracle(160)
    s = UnsSolver(_uns_case(), mesh_text=meshgen.hmshb_bytes(verts, codes))
    s.set_state(_uns_toro_state(verts))
    s.run(steps)
    np.testing.assert_array_equal(s.state(), U)
    assert s.time()[0] == t
