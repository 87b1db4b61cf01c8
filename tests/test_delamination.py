"""Flat-shell delamination topology (split_delam_nodes_flat_shell.m) on CPU.

The product's vectorised splitter must reproduce the oracle's literal
restatement of the reference loops exactly (node ids, coordinates, element
lists) on interior, edge, corner, L-shaped, single-element, empty and
whole-plate zones.  A physical identity pins the sub-laminates: with every
split copy moved like its original, the delaminated plate's K*U, folded back
onto the original nodes, equals the intact plate's (above + under = intact
laminate, integrated about the same mid-plane).
"""
import numpy as np
import pytest

from oracle import ref_setup as R
from oracle.oracle import OracleProblem


def _cases(pkg):
    MS = pkg.mesh
    mesh = MS.structured_plate(0.12, 0.1, 12, 10)
    nex = 12
    el = lambda ix, iy: iy * nex + ix
    return mesh, {
        "interior_ellipse": MS.elements_in_ellipse(mesh, 0.06, 0.05, 0.035, 0.02, 0.3),
        "touches_left_edge": np.array([el(0, 4), el(1, 4), el(0, 5), el(1, 5), el(2, 5)]),
        "plate_corner": np.array([el(0, 0), el(1, 0), el(0, 1), el(1, 1)]),
        "l_shape": np.array([el(4, 4), el(5, 4), el(6, 4), el(4, 5), el(4, 6)]),
        "single": np.array([el(7, 3)]),
        "strip_across": np.array([el(i, 2) for i in range(nex)]),
        "empty": np.zeros(0, np.int64),
        "whole_plate": np.arange(120),
        "two_corners_on_edge": np.array([el(5, 0), el(6, 0)]),
    }


@pytest.mark.parametrize("name", ["interior_ellipse", "touches_left_edge", "plate_corner", "l_shape", "single",
                                  "strip_across", "empty", "whole_plate", "two_corners_on_edge"])
def test_splitter_matches_reference_loops(pkg, name):
    mesh, cases = _cases(pkg)
    den = cases[name]
    bn = pkg.mesh.boundary_nodes(mesh)
    n1, c1, du, da = pkg.mesh.split_delam_nodes_flat_shell(mesh["nodes"], mesh["coords"], den, bn)
    n2, c2, du2, da2 = R.split_delam_nodes_flat_shell(mesh["nodes"], mesh["coords"], den + 1, 6, 6, bn)
    assert np.array_equal(n1, n2)
    assert np.array_equal(c1, c2)
    assert list(du + 1) == du2 and list(da + 1) == da2
    fen = mesh["nodes"].shape[0]
    assert np.array_equal(n1[:fen], mesh["nodes"])           # intact rows and den_under keep their nodes
    if len(den):
        new = n1[da] > mesh["coords"].shape[0]
        assert np.array_equal(c1[n1[da][new] - 1], c1[mesh["nodes"][den][new] - 1])
        assert c1.shape[0] == mesh["coords"].shape[0] + np.unique(n1[da][new]).size


def test_interior_zone_keeps_perimeter_shared(pkg):
    mesh, cases = _cases(pkg)
    den = cases["interior_ellipse"]
    n1, c1, du, da = pkg.mesh.split_delam_nodes_flat_shell(mesh["nodes"], mesh["coords"], den,
                                                           pkg.mesh.boundary_nodes(mesh))
    fen = mesh["nodes"].shape[0]
    rest = np.setdiff1d(np.arange(fen), den)
    shared = np.intersect1d(n1[da], n1[du])
    # exactly the zone's perimeter is shared: every shared node is also used by an intact element
    assert shared.size > 0 and np.all(np.isin(shared, n1[rest]))
    # and every node of the zone that an intact element uses is shared, except
    # the concave corners of the staircase zone (corner of three delaminated
    # elements), which the reference's corner rule splits
    zone_nodes = np.unique(n1[du])
    unshared = np.setdiff1d(np.intersect1d(zone_nodes, n1[rest]), shared)
    corners = mesh["nodes"][den][:, [0, 5, 30, 35]].reshape(-1)
    assert all((corners == x).sum() == 3 for x in unshared)
    assert unshared.size < shared.size


def _sub_tables(pkg, layer):
    M = pkg.materials
    q = M.ply_stiffness(**M.CFRP_PLY)
    full = M.laminate(q, M.CFRP_RHO, M.CFRP_PLY_T, M.CFRP_ANGLES)
    ab = M.laminate(q, M.CFRP_RHO, M.CFRP_PLY_T, M.CFRP_ANGLES, plies=range(layer))
    un = M.laminate(q, M.CFRP_RHO, M.CFRP_PLY_T, M.CFRP_ANGLES, plies=range(layer, 8))
    return np.stack([M.table_row(full), M.table_row(ab), M.table_row(un)])


def test_sub_laminates_add_up_to_intact(pkg):
    """above + under == intact for every ABD, shear and mass term (same
    mid-plane, same shear-correction thickness; the oracle's sub-laminate
    formulas are pinned in test_oracle_setup)."""
    K = pkg.materials.ABD_KEYS
    for layer in (1, 3, 4, 7):
        full, ab, un = _sub_tables(pkg, layer)
        for k, f, x, y in zip(K, full, ab, un):
            assert abs(x + y - f) <= 1e-12 * max(abs(f), abs(x), abs(y), 1e-300), k


def test_split_stiffness_folds_to_intact(pkg):
    mesh, cases = _cases(pkg)
    den = cases["interior_ellipse"]
    n1, c1, du, da = pkg.mesh.split_delam_nodes_flat_shell(mesh["nodes"], mesh["coords"], den,
                                                           pkg.mesh.boundary_nodes(mesh))
    tab = _sub_tables(pkg, 3)
    em = np.zeros(n1.shape[0], np.int32)
    em[du], em[da] = 2, 1
    nn0 = mesh["coords"].shape[0]
    nn1 = c1.shape[0]
    # original of every node (copies map back onto the node they split from)
    orig = np.arange(nn1)
    orig[n1[da].reshape(-1) - 1] = mesh["nodes"][den].reshape(-1) - 1
    rng = np.random.default_rng(5)
    U0 = rng.standard_normal(5 * nn0)
    U1 = U0.reshape(nn0, 5)[orig].reshape(-1)
    K0 = OracleProblem(mesh["nodes"], mesh["coords"], tab[:1]).apply_k(U0)
    K1 = OracleProblem(n1, c1, tab, em).apply_k(U1)
    folded = np.zeros((nn0, 5))
    np.add.at(folded, orig, K1.reshape(nn1, 5))
    assert np.linalg.norm(folded.reshape(-1) - K0) <= 1e-12 * np.linalg.norm(K0)
    # and the split copies do carry force of their own (the plies are disconnected there)
    assert np.abs(K1.reshape(nn1, 5)[nn0:]).max() > 0
