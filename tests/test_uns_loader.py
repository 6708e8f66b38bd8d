"""The unstructured loader's neighbour search (hf_uns_mesh_neighbours: the product's C++ loader,
run on the host, no GPU) against the reference's own loader, LoadStructuredMesh
(src/fvm_2d_uns/mesh/mesh_structured/mesh_structured.cpp:92-114), whose rule is
Edge::opposite_edges_equal within 1e-12 per coordinate (src/fvm_2d_uns/geometry/edge/edge.cpp:59-71)
with the last match in pair order winning.

The fixtures hold the reference loader's cell_edge_indices for meshes the reference's own
generator (src/mesh_generation/generate_block_mesh.py) made from its scramjet case: there
neighbouring cells' shared vertices differ in their last bits, so an exact-coordinate match
leaves a third of the interior pairs unmatched.  The small hand-made meshes below probe the
tolerance's edges; where the reference build is present (oracle/_ref) they also run through the
reference loader itself."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _neighbours(V, codes):
    from hyperflow_gb300 import meshgen, uns
    return uns.mesh_neighbours(meshgen.hmsh_text(V, codes))


def _ref_loader(V, codes, tmp_path):
    """the reference's own LoadStructuredMesh on this quad mesh, or None without the build"""
    from hyperflow_gb300 import meshgen
    from oracle import oracle
    if not os.path.exists(oracle.REF_UNS_LIB):
        return None
    path = tmp_path / "mesh.hmsh"
    path.write_text(meshgen.hmsh_text(V, codes))
    case = meshgen.channel_case(str(path))
    case["mesh"]["type"] = "hyperflow_structured"
    return oracle.RefUns.from_file(case).nbr


def _exact_matches(V):
    """pairs whose reversed edge occurs with bit-identical coordinates"""
    S = V.reshape(-1, 2)
    nv = V.shape[1]
    nxt = np.arange(len(S)) + 1
    nxt[nv - 1::nv] -= nv
    keys = {(a, b, c, d) for a, b, c, d in zip(S[:, 0], S[:, 1], S[nxt, 0], S[nxt, 1])}
    return sum((c, d, a, b) in keys for a, b, c, d in zip(S[:, 0], S[:, 1], S[nxt, 0], S[nxt, 1]))


def test_loader_equals_reference_loader_on_scramjet_coarse():
    """The reference's scramjet coarse mesh (22,960 quads): every one of the 91,840 pairs gets
    the reference loader's neighbour -- all 90,832 interior pairs matched, where bit-exact
    coordinates match only 59,210."""
    from oracle import oracle
    g = np.load(os.path.join(GOLDEN, "loader_scramjet_coarse.npz"))
    V, codes, ref = g["verts"], g["codes"].astype(np.int32), g["nbr"]
    nbr, unmatched, first = _neighbours(V, codes)
    np.testing.assert_array_equal(nbr, ref)
    assert unmatched == 0 and first == -1
    interior = int((codes >= 0).sum())
    assert interior == 90_832 and len(ref) == 91_840
    assert _exact_matches(V) == 59_210           # the tolerance decides a third of the pairs
    np.testing.assert_array_equal(oracle.ref_neighbours(V, codes)[0], ref)   # the oracle's restatement


@pytest.mark.parametrize("name", ["scramjet_reduced4", "quad_channel_240", "tri_hole_3k"])
def test_loader_equals_fixture_neighbours(name):
    g = np.load(os.path.join(GOLDEN, f"uns_{name}.npz"))
    nbr, unmatched, _ = _neighbours(g["verts"], g["codes"])
    np.testing.assert_array_equal(nbr, g["nbr"])
    assert unmatched == 0


def _two_quads(dx=0.0, dy=0.0):
    """two unit quads sharing the edge x = 1; the right quad's shared vertices moved by (dx, dy)"""
    a = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)]
    b = [(1.0 + dx, 0.0 + dy), (2.0, 0.0), (2.0, 1.0), (1.0 + dx, 1.0 + dy)]
    return np.array([a, b]), np.array([[-1, 0, -1, -3], [-1, -2, -1, 0]], np.int32)


@pytest.mark.parametrize("d,matched", [(0.0, True), (0.9e-12, True), (-0.9e-12, True),
                                       (1.1e-12, False), (-1.1e-12, False), (5e-13, True)])
def test_tolerance_edge(d, matched, tmp_path):
    """within 1e-12 (strictly) per coordinate the edges meet; beyond, the interior pairs keep
    code 0 -- cell 0 -- and are reported"""
    for dx, dy in ((d, 0.0), (0.0, d), (d, d)):
        V, codes = _two_quads(dx, dy)
        nbr, unmatched, first = _neighbours(V, codes)
        if matched:
            assert nbr[1] == 1 and nbr[7] == 0 and unmatched == 0
        else:
            assert nbr[1] == 0 and nbr[7] == 0 and unmatched == 2 and first == 1
        ref = _ref_loader(V, codes, tmp_path)
        if ref is not None:
            np.testing.assert_array_equal(nbr, ref)


def test_last_match_wins_and_degenerate_edges(tmp_path):
    """A cell repeated three times: each pair of the first copy takes the LAST copy as its
    neighbour (the reference's scan keeps the last match).  A quad with two coincident vertices
    has an edge of zero length, which equals itself reversed: its neighbour is its own cell."""
    from oracle import oracle
    a = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)]
    b = [(1.0, 1.0), (1.0, 0.0), (2.0, 0.0), (2.0, 1.0)]            # shares a's right edge reversed
    deg = [(3.0, 0.0), (4.0, 0.0), (4.0, 1.0), (4.0, 1.0)]           # zero-length third edge
    V = np.array([a, b, b, b, deg])
    codes = np.zeros((5, 4), np.int32)
    nbr, _, _ = _neighbours(V, codes)
    assert nbr[1] == 3                      # a's right edge: the last of the three copies
    assert nbr[4 * 4 + 2] == 4              # the degenerate edge matches itself
    np.testing.assert_array_equal(nbr, oracle.ref_neighbours(V, codes)[0])
    ref = _ref_loader(V, codes, tmp_path)
    if ref is not None:
        np.testing.assert_array_equal(nbr, ref)


def test_grid_lines_large_and_non_finite_coordinates(tmp_path):
    """Shared vertices that straddle a line of the loader's hash grid (multiples of 2^-30) still
    meet; beyond 2^32 a coordinate's ulp exceeds the tolerance, so only equal values meet; a NaN
    vertex meets nothing and breaks nothing."""
    from oracle import oracle
    g = 2.0 ** -30
    x = 7 * g
    left = [(0.0, 0.0), (x, 0.0), (x, 1.0), (0.0, 1.0)]
    right = [(x - 4e-13, 0.0), (1.0, 0.0), (1.0, 1.0), (x - 4e-13, 1.0)]   # across the grid line
    big = 2.0 ** 33
    bl = [(big, 0.0), (big + 2.0, 0.0), (big + 2.0, 1.0), (big, 1.0)]
    br = [(big + 2.0, 0.0), (big + 4.0, 0.0), (big + 4.0, 1.0), (big + 2.0, 1.0)]
    nan = [(5.0, 5.0), (float("nan"), 5.0), (6.0, 6.0), (5.0, 6.0)]
    V = np.array([left, right, bl, br, nan])
    codes = np.zeros((5, 4), np.int32)
    nbr, unmatched, _ = _neighbours(V, codes)
    assert nbr[1] == 1 and nbr[7] == 0     # across the grid line
    assert nbr[9] == 3 and nbr[15] == 2    # large, equal coordinates
    np.testing.assert_array_equal(nbr, oracle.ref_neighbours(V, codes)[0])
    ref = _ref_loader(V, codes, tmp_path)
    if ref is not None:
        np.testing.assert_array_equal(nbr, ref)


def test_unmatched_pairs_reported_by_solver_api_shape():
    """hf_uns_unmatched_pairs is exported; the host-only loader reports the same numbers as the
    oracle's restatement on a mesh with a gap."""
    from hyperflow_gb300 import _lib
    from oracle import oracle
    assert hasattr(_lib.lib(), "hf_uns_unmatched_pairs")
    V, codes = _two_quads(3e-12, 0.0)
    nbr, unmatched, first = _neighbours(V, codes)
    onbr, oun = oracle.ref_neighbours(V, codes)
    np.testing.assert_array_equal(nbr, onbr)
    assert unmatched == oun == 2
