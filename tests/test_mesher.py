"""Mesh input path: gmsh's MATLAB export, quad orientation, quad ->
spectral conversion (quad2spectral_Fiborek.m numbering), against the oracle's
restatement of the reference's steps."""
import numpy as np
import pytest

from oracle import ref_setup as R


def jittered_quads(nx=6, ny=5, Lx=0.1, Ly=0.08, amp=0.004, seed=0, flip=(3,), angle=0.0):
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.linspace(0, Lx, nx), np.linspace(0, Ly, ny))
    pos = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1)
    inner = (pos[:, 0] > 0) & (pos[:, 0] < Lx) & (pos[:, 1] > 0) & (pos[:, 1] < Ly)
    pos[inner, :2] += rng.uniform(-amp, amp, (inner.sum(), 2))
    if angle:
        c, s = np.cos(angle), np.sin(angle)
        pos[:, :2] = pos[:, :2] @ np.array([[c, s], [-s, c]])
    q = np.array([[j * nx + i + 1, j * nx + i + 2, (j + 1) * nx + i + 2, (j + 1) * nx + i + 1]
                  for j in range(ny - 1) for i in range(nx - 1)])
    for f in flip:
        q[f] = q[f][[0, 3, 2, 1]]   # clockwise
    return q, pos


@pytest.mark.parametrize("order", [5, 4])
@pytest.mark.parametrize("seed,angle", [(0, 0.0), (1, 0.7), (2, -2.1)])
def test_quad2spectral_matches_reference_steps(pkg, order, seed, angle):
    q, pos = jittered_quads(seed=seed, angle=angle, flip=(3, 7))
    q1 = pkg.mesher.change_turn_quad(q, pos)
    q2 = R.change_turn_quad(q, pos)
    assert np.array_equal(q1, q2) and (q1 != q).any(axis=1).sum() == 2
    n1, c1, b1 = pkg.mesher.quad2spectral(q1, pos, order)
    n2, c2, b2 = R.quad2spectral_fiborek(q2, pos, order)
    assert np.array_equal(n1, n2)
    assert np.abs(c1 - c2).max() <= 1e-15
    assert np.array_equal(b1, b2)
    n = order + 1
    assert c1.shape[0] == (5 * order + 1) * (4 * order + 1) and n1.shape == (20, n * n)
    # every node is used; element corners keep the quad numbers
    assert np.array_equal(np.unique(n1), np.arange(1, c1.shape[0] + 1))
    assert np.array_equal(n1[:, [0, n - 1, n * n - 1, n * n - n]], q1)


def test_quad2spectral_of_a_regular_grid_is_the_structured_node_set(pkg):
    q, pos = jittered_quads(amp=0.0, flip=())
    nodes, coords, bnd = pkg.mesher.quad2spectral(q, pos, 5)
    ref = pkg.mesh.structured_plate(0.1, 0.08, 5, 4)
    a = np.round(coords[:, :2], 12)
    b = np.round(ref["coords"][:, :2], 12)
    assert np.array_equal(a[np.lexsort(a.T[::-1])], b[np.lexsort(b.T[::-1])])
    on_edge = (np.isclose(coords[:, 0], 0) | np.isclose(coords[:, 0], 0.1) | np.isclose(coords[:, 1], 0) |
               np.isclose(coords[:, 1], 0.08))
    assert np.array_equal(np.sort(bnd), np.nonzero(on_edge)[0] + 1)


def test_read_gmsh_matlab_export(pkg, tmp_path):
    q, pos = jittered_quads(nx=3, ny=3, flip=())
    f = tmp_path / "plate.m"
    with open(f, "w") as fh:
        fh.write(f"msh.nbNod = {pos.shape[0]};\n")
        fh.write("msh.POS = [\n" + "".join(f"{x:.15g} {y:.15g} {z:.15g};\n" for x, y, z in pos) + "];\n")
        fh.write("msh.MAX = [0.1 0.08 0];\nmsh.MIN = [0 0 0];\n")
        fh.write("msh.QUADS = [\n" + "".join(f" {a} {b} {c} {d} {1 + (k % 2)}\n" for k, (a, b, c, d) in
                                             enumerate(q)) + "];\n")
    m = pkg.mesher.read_gmsh_m(str(f))
    assert m["nbNod"] == pos.shape[0]
    assert np.allclose(m["POS"], pos, rtol=0, atol=1e-15)
    assert np.array_equal(m["QUADS"][:, :4].astype(int), q) and set(m["QUADS"][:, 4]) == {1.0, 2.0}
    assert np.array_equal(m["MAX"], [[0.1, 0.08, 0.0]])
