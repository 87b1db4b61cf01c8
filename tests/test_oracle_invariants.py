"""Invariants of the oracle's stiffness operators that any correct restatement
must have (CPU only), on distorted meshes with several materials: rigid-body
fields produce no force, K is symmetric and positive semi-definite.

Isoparametric elements reproduce every field that is linear in x, y (and z)
exactly, so a rigid translation or rotation has zero strain at every GLL
node, whatever the element shape.  Flat shell, DOF order (u, phi_x, v,
phi_y, w): the in-plane rotation u = -y, v = x has no membrane strain, and the
tilt w = x with phi_x = -1 (w = y with phi_y = -1) has neither curvature nor
transverse shear (the reference's shear strains are phi_x + dw/dx and
phi_y + dw/dy).  3D solid, DOF order (u, v, w): three translations and the
three rotations."""
import numpy as np
import pytest

from oracle.oracle import OracleProblem, OracleSolid
from test_oracle_physics import _distorted, _materials

RIGID_TOL = 1e-9   # |K r| / |K u| for a rigid field r and a random field u of the same norm
SYM_TOL = 1e-12


def _shell_problem(pkg):
    mesh = _distorted(pkg, nex=3, ney=2, seed=4)
    lams = _materials(pkg)
    fen = mesh["nodes"].shape[0]
    elem_mat = np.arange(fen) % 2
    keep = np.linspace(0.5, 1.0, fen)
    table = np.stack([pkg.materials.table_row(l) for l in lams])
    return mesh, OracleProblem(mesh["nodes"], mesh["coords"], table, elem_mat, keep)


def _solid_problem(pkg):
    scs, _ = pkg.workloads.solid_plate(nex=3, L=0.015, T=2e-6, f=800e3, n_out=2, radius=0.004, delam=False)
    sc = scs[0]
    c = sc.mesh["coords"].copy()
    base = sc.mesh["base"]["coords"]
    L = base[:, 0].max()
    inner = (base[:, 0] > 0) & (base[:, 0] < L) & (base[:, 1] > 0) & (base[:, 1] < L)
    jit = np.zeros((base.shape[0], 2))
    jit[inner] = np.random.default_rng(3).uniform(-0.04, 0.04, (inner.sum(), 2)) * (L / 3 / 5)
    nxy = base.shape[0]
    for k in range(c.shape[0] // nxy):
        c[k * nxy:(k + 1) * nxy, :2] += jit
    fen = sc.mesh["nodes"].shape[0]
    keep = np.linspace(0.6, 1.0, fen)
    return c, OracleSolid(sc.mesh["nodes"], c, sc.mat_table[:, :13], sc.mat_table[:, 13], sc.elem_mat, keep)


def _rigid_ratio(apply_k, rigid, n, seed):
    u = np.random.default_rng(seed).standard_normal(n)
    ku = np.linalg.norm(apply_k(u / np.linalg.norm(u)))
    return [np.linalg.norm(apply_k(r / np.linalg.norm(r))) / ku for r in rigid]


def test_shell_rigid_fields_give_no_force(pkg):
    mesh, orc = _shell_problem(pkg)
    x, y = mesh["coords"][:, 0], mesh["coords"][:, 1]
    nn = x.size

    def field(**comp):
        U = np.zeros((nn, 5))
        for k, v in comp.items():
            U[:, "u phix v phiy w".split().index(k)] = v
        return U.reshape(-1)
    rigid = [field(u=1.0), field(v=1.0), field(w=1.0), field(u=-y, v=x),
             field(w=x, phix=-1.0), field(w=y, phiy=-1.0)]
    ratios = _rigid_ratio(orc.apply_k, rigid, 5 * nn, seed=1)
    assert max(ratios) <= RIGID_TOL, ratios
    # a field that bends does produce force
    assert _rigid_ratio(orc.apply_k, [field(w=x * x)], 5 * nn, seed=1)[0] > 1e-6


def test_solid_rigid_fields_give_no_force(pkg):
    c, orc = _solid_problem(pkg)
    x, y, z = c[:, 0], c[:, 1], c[:, 2]
    nn = x.size
    one, zero = np.ones(nn), np.zeros(nn)

    def field(u, v, w):
        return np.stack([u, v, w], axis=1).reshape(-1)
    rigid = [field(one, zero, zero), field(zero, one, zero), field(zero, zero, one),
             field(-y, x, zero), field(zero, -z, y), field(z, zero, -x)]
    ratios = _rigid_ratio(orc.apply_k, rigid, 3 * nn, seed=2)
    assert max(ratios) <= RIGID_TOL, ratios
    assert _rigid_ratio(orc.apply_k, [field(x * x, zero, zero)], 3 * nn, seed=2)[0] > 1e-6


@pytest.mark.parametrize("which", ["shell", "solid"])
def test_stiffness_symmetric_positive_semidefinite(pkg, which):
    _, orc = _shell_problem(pkg) if which == "shell" else _solid_problem(pkg)
    n = orc.ndof
    rng = np.random.default_rng(7)
    for _ in range(3):
        u, v = rng.standard_normal(n), rng.standard_normal(n)
        ku, kv = orc.apply_k(u), orc.apply_k(v)
        scale = np.linalg.norm(ku) * np.linalg.norm(v)
        assert abs(v @ ku - u @ kv) <= SYM_TOL * scale
        assert u @ ku > 0 and v @ kv > 0
