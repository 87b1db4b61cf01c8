"""The oracle's time loop against an independent dense derivation and physics
invariants (CPU only).  Two derivations must agree before the GPU is trusted:
the oracle's literal restatement of main_flat_shell.m (sparse derivative
blocks, 12-basket scatter) and a B^T C B element-matrix assembly."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle.oracle import OracleProblem


def _distorted(pkg, nex=3, ney=2, seed=1, amp=0.15):
    """Structured plate whose element corners are jittered (curved-free, straight edges)."""
    m = pkg.mesh.structured_plate(0.03, 0.02, nex, ney)
    rng = np.random.default_rng(seed)
    ax, ay = m["ax"], m["ay"]
    # move each element-corner grid point, interpolate interior nodes bilinearly
    cx = np.arange(nex + 1) * ax
    cy = np.arange(ney + 1) * ay
    CX, CY = np.meshgrid(cx, cy)
    CX[1:-1, 1:-1] += rng.uniform(-amp, amp, CX[1:-1, 1:-1].shape) * ax
    CY[1:-1, 1:-1] += rng.uniform(-amp, amp, CY[1:-1, 1:-1].shape) * ay
    x, _ = pkg.mesh.gll_points(6)
    s = (x + 1) / 2
    coords = m["coords"].copy()
    for ey in range(ney):
        for ex in range(nex):
            for k in range(6):
                for i in range(6):
                    g = m["nodes"][ey * nex + ex, k * 6 + i] - 1
                    a, b = s[i], s[k]
                    px = (1 - a) * (1 - b) * CX[ey, ex] + a * (1 - b) * CX[ey, ex + 1] + \
                        (1 - a) * b * CX[ey + 1, ex] + a * b * CX[ey + 1, ex + 1]
                    py = (1 - a) * (1 - b) * CY[ey, ex] + a * (1 - b) * CY[ey, ex + 1] + \
                        (1 - a) * b * CY[ey + 1, ex] + a * b * CY[ey + 1, ex + 1]
                    coords[g, 0], coords[g, 1] = px, py
    m = dict(m)
    m["coords"] = coords
    return m


def _materials(pkg):
    M = pkg.materials
    q = M.ply_stiffness(130e9, 10e9, 0.3, 5e9, 5e9, 3.5e9)
    lam0 = M.laminate(q, 1570.0, [0.4875e-3] * 8, (0, 90, 45, -45, -45, 45, 90, 0))
    lam1 = M.laminate(q, 1570.0, [0.4875e-3] * 4, (30, -60, 15, 70))  # unsymmetric: B != 0
    return [lam0, lam1]


def _dense_K(pkg, mesh, lams, elem_mat, keep):
    E = pkg.element
    nodes = mesh["nodes"]
    nn = mesh["coords"].shape[0]
    rows, cols, vals = [], [], []
    for e in range(nodes.shape[0]):
        xy = mesh["coords"][nodes[e] - 1, :2]
        Ke = E.element_stiffness(xy, lams[elem_mat[e]]) * keep[e]
        dofs = (5 * (nodes[e] - 1)[:, None] + np.arange(5)[None, :]).reshape(-1)
        rows.append(np.repeat(dofs, len(dofs)))
        cols.append(np.tile(dofs, len(dofs)))
        vals.append(Ke.reshape(-1))
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(5 * nn, 5 * nn))


@pytest.mark.parametrize("distort", [False, True])
def test_oracle_stiffness_equals_dense_assembly(pkg, distort):
    mesh = _distorted(pkg) if distort else pkg.mesh.structured_plate(0.03, 0.02, 3, 2)
    lams = _materials(pkg)
    fen = mesh["nodes"].shape[0]
    elem_mat = np.arange(fen) % 2
    keep = np.linspace(0.4, 1.0, fen)
    table = np.stack([pkg.materials.table_row(l) for l in lams])
    orc = OracleProblem(mesh["nodes"], mesh["coords"], table, elem_mat, keep)
    K = _dense_K(pkg, mesh, lams, elem_mat, keep)
    rng = np.random.default_rng(3)
    for _ in range(3):
        U = rng.standard_normal(5 * mesh["coords"].shape[0]) * 1e-9
        F = orc.apply_k(U)
        Fd = K @ U
        assert np.linalg.norm(F - Fd) <= 1e-11 * np.linalg.norm(Fd)
    # symmetric, with the rigid-body modes in its null space
    Kd = K.toarray()
    assert np.abs(Kd - Kd.T).max() <= 1e-9 * np.abs(Kd).max()
    x = mesh["coords"][:, 0]
    for mode in range(4):
        U = np.zeros(5 * len(x))
        if mode < 3:
            U[[0, 2, 4][mode]::5] = 1e-6          # translations u, v, w
        else:
            U[4::5] = -1e-6 * x                   # rotation: w = -theta x, phi_x = theta
            U[1::5] = 1e-6
        F = orc.apply_k(U)
        assert np.abs(F).max() <= 1e-9 * np.abs(Kd).max() * 1e-6 * 36


def test_oracle_time_loop_equals_dense_loop(pkg):
    """Oracle MAIN LOOP == a dense-matrix central-difference loop (reference update)."""
    W = pkg.workloads
    scs, run = W.plate_force(nex=3, ney=3, L=0.03, T=3e-6)
    sc = scs[0]
    lam = pkg.materials.cfrp_laminate()
    orc = OracleProblem(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table)
    res = orc.run(run.dt, run.nft, sc.signal, nn_first=run.nn_first, eta_xy=run.eta_xy, eta_z=run.eta_z,
                  force_dof=sc.force_dof, force_val=sc.force_val, out_dof=sc.out_dof, h=run.h)
    K = _dense_K(pkg, sc.mesh, [lam], np.zeros(9, int), np.ones(9))
    a0, a1, mgs, mg2, mg0, cg = orc.coefficients(run.dt, run.eta_xy, run.eta_z)
    n = K.shape[0]
    U = np.zeros(n)
    Uo = np.zeros(n)
    Fa = np.zeros(n)
    Fa[sc.force_dof - 1] = sc.force_val
    displ = np.zeros((run.nft, len(sc.out_dof)))
    for nn in range(run.nn_first, run.nft + 1):
        F = -(K @ U) + mg2 * U + Fa * sc.signal[nn - 1] - mgs * Uo + a1 * cg * Uo
        un = mg0 * F
        displ[nn - 1] = U[sc.out_dof - 1]
        Uo, U = U, un
    assert np.max(np.abs(res["displ"])) > 0
    assert np.linalg.norm(res["displ"] - displ) <= 1e-10 * np.linalg.norm(displ)
    assert np.linalg.norm(res["U"] - U) <= 1e-10 * np.linalg.norm(U)


def test_oracle_energy_conserved_without_damping(pkg):
    """Undamped central difference conserves the discrete energy
    E_n+1/2 = 1/2 v'Mv + 1/2 u_n+1' K u_n after the load ends."""
    W = pkg.workloads
    scs, run = W.plate_force(nex=2, ney=2, L=0.02, T=40e-6, f=400e3)
    sc = scs[0]
    orc = OracleProblem(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table)
    mg = orc.mg_raw
    energies = []
    U = Uo = None
    nn = run.nn_first
    stride = 40
    for stop in range(run.nn_first + stride, run.nft, stride):
        r = orc.run(run.dt, run.nft, sc.signal, nn_first=nn, force_dof=sc.force_dof, force_val=sc.force_val,
                    U0=U, uold0=Uo, nn_last=stop - 1)
        U, Uo, nn = r["U"], r["uold"], stop
        if sc.signal[nn - 2:].any():
            continue
        v = (U - Uo) / run.dt
        energies.append(0.5 * v @ (mg * v) + 0.5 * U @ orc.apply_k(Uo))
    energies = np.array(energies)
    assert len(energies) >= 3 and energies[0] > 0
    assert np.max(np.abs(energies - energies[0])) <= 1e-8 * energies[0]
