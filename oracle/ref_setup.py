"""Oracle, setup half: FP64 NumPy restatement of ma-shm's flat-shell set-up.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
it, and only as the test oracle (or as the timed CPU reference arm).

Every function restates one file of the reference (paths are relative to the
ma-shm repository) in the same arithmetic order, deliberately literal: loops
where the MATLAB code loops, the same intermediate quantities, the same
thresholds.  The time loop itself lives in ``sem_oracle.c``.
"""
from __future__ import annotations

import numpy as np

# --------------------------------------------------------------------------
# element math
# --------------------------------------------------------------------------


def gll(n: int):
    """GLL nodes and weights, ``src/models/flat_shell/flat_shell_engine/gll.m:1-39``.

    gll.m hard-codes a table for n = 2..10.  The oracle recomputes the same
    numbers from their definition (interior nodes = roots of P'_{n-1}, weights
    2 / (n (n-1) P_{n-1}(x)^2)) with a Newton polish; the tests pin the result
    against the table printed in gll.m (tests/golden/gll_ref.json).
    """
    if n == 1:
        return np.zeros(1), np.ones(1)
    if n == 2:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    leg = np.polynomial.legendre.Legendre.basis(n - 1)
    dleg = leg.deriv()
    ddleg = dleg.deriv()
    inner = np.sort(dleg.roots().real)
    for _ in range(6):  # Newton polish on P'_{n-1}
        inner = inner - dleg(inner) / ddleg(inner)
    x = np.concatenate(([-1.0], inner, [1.0]))
    # symmetrise exactly like the table (ksi(k) = -ksi(n+1-k))
    x = 0.5 * (x - x[::-1])
    w = 2.0 / (n * (n - 1) * leg(x) ** 2)
    w = 0.5 * (w + w[::-1])
    return x, w


def vandermonde(ksi: np.ndarray) -> np.ndarray:
    """``flat_shell_engine/Vandermonde.m:6-12``: V(i,j) = ksi(j)^(i-1); Q = inv(V)."""
    n = len(ksi)
    V = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            V[i, j] = ksi[j] ** i
    return np.linalg.inv(V)


def shape2d_prim(nx: int, ny: int, Qx, Qy, x, y):
    """``flat_shell_engine/shape2D_prim.m:10-58``.

    Returns the element blocks Nprimx, Nprimy (nx*ny square) of the sparse
    derivative operators Npx, Npy; node/shape numbering c = (k2-1)*nx + k1
    (xi fastest) and entries with |v| < 1e-12 set to 0 exactly as the
    reference does.
    """
    ux = np.zeros((nx, nx))
    uy = np.zeros((ny, ny))
    ux[:, 0] = 1.0
    uy[:, 0] = 1.0
    for j in range(1, nx):
        ux[:, j] = x ** j
    for j in range(1, ny):
        uy[:, j] = y ** j
    Sx = ux @ Qx.T
    Sy = uy @ Qy.T
    uxp = np.zeros((nx, nx))
    uyp = np.zeros((ny, ny))
    for j in range(1, nx):
        uxp[:, j] = j * x ** (j - 1)
    for j in range(1, ny):
        uyp[:, j] = j * y ** (j - 1)
    Sxp = uxp @ Qx.T
    Syp = uyp @ Qy.T
    Nx = np.zeros((nx * ny, nx * ny))
    Ny = np.zeros((nx * ny, nx * ny))
    c = 0
    for k2 in range(ny):
        for k1 in range(nx):
            cc = 0
            for j2 in range(ny):
                for j1 in range(nx):
                    vx = Sxp[k1, j1] * Sy[k2, j2]
                    vy = Sx[k1, j1] * Syp[k2, j2]
                    Nx[c, cc] = 0.0 if abs(vx) < 1e-12 else vx
                    Ny[c, cc] = 0.0 if abs(vy) < 1e-12 else vy
                    cc += 1
            c += 1
    return Nx, Ny


def sparse_pattern(N: np.ndarray):
    """MATLAB ``[i,j]=find(N)`` order (column-major), 0-based, plus values
    (``main_flat_shell.m:267-281``)."""
    cols, rows = np.nonzero(N.T)  # transpose => column-major enumeration
    return rows.astype(np.int32), cols.astype(np.int32), N[rows, cols].copy()


def jacobians(nodes1: np.ndarray, coords: np.ndarray, Nprimx, Nprimy):
    """``main_flat_shell.m:309-350`` + ``inv_jacp_2D.m:3-8`` + ``det_jacp_2D.m:3``.

    nodes1: [fen, 36] 1-based.  Returns per-local-node arrays (length
    fen*36, element-major) J11, J21, J12, J22, invJ11, invJ12, invJ21,
    invJ22, detJ.
    """
    X = coords[nodes1 - 1, 0]  # [fen,36]
    Y = coords[nodes1 - 1, 1]
    J11 = X @ Nprimx.T  # Npx*X, per element block
    J21 = Y @ Nprimx.T
    J12 = X @ Nprimy.T
    J22 = Y @ Nprimy.T
    a = 1.0 / (J11 * J22 - J12 * J21)
    invJ11 = a * J22
    invJ12 = a * (-J12)
    invJ21 = a * (-J21)
    invJ22 = a * J11
    detJ = J11 * J22 - J12 * J21
    f = lambda v: np.ascontiguousarray(v.reshape(-1))
    return dict(J11=f(J11), J21=f(J21), J12=f(J12), J22=f(J22),
                invJ11=f(invJ11), invJ12=f(invJ12), invJ21=f(invJ21),
                invJ22=f(invJ22), detJ=f(detJ))


def quad_weights(nx: int, ny: int, wx, wy):
    """``main_flat_shell.m:400-410``: ww(cc) = wx(kx)*wy(ky), kx fastest."""
    ww = np.zeros(nx * ny)
    cc = 0
    for ky in range(ny):
        for kx in range(nx):
            ww[cc] = wx[kx] * wy[ky]
            cc += 1
    return ww


# --------------------------------------------------------------------------
# materials
# --------------------------------------------------------------------------


def ply_z(lh):
    """Ply z-ranges from the top surface downward (``lay_const.m:16-21``)."""
    lay = len(lh)
    h = float(np.sum(lh))
    h2 = np.zeros(lay)
    h1 = np.zeros(lay)
    h2[0] = h / 2
    h1[0] = h / 2 - lh[0]
    for i in range(1, lay):
        h2[i] = h2[i - 1] - lh[i - 1]
        h1[i] = h1[i - 1] - lh[i]
    return h, h1, h2


def rotated_q(q11, q12, q22, q44, q55, q66, alpha_deg):
    """Rotated ply stiffness, ``composite_plate_c_delam.m:8-20``."""
    ar = np.asarray(alpha_deg, dtype=float) * np.pi / 180
    m = np.cos(ar)
    n = np.sin(ar)
    s11 = q11 * m**4 + 2 * (q12 + 2 * q66) * m**2 * n**2 + q22 * n**4
    s12 = (q11 + q22 - 4 * q66) * m**2 * n**2 + q12 * (m**4 + n**4)
    s16 = (q11 - q12 - 2 * q66) * m**3 * n + (q12 - q22 + 2 * q66) * m * n**3
    s22 = q11 * n**4 + 2 * (q12 + 2 * q66) * m**2 * n**2 + q22 * m**4
    s26 = (q11 - q12 - 2 * q66) * n**3 * m + (q12 - q22 + 2 * q66) * n * m**3
    s44 = q44 * m**2 + q55 * n**2
    s45 = (q55 - q44) * m * n
    s55 = q55 * m**2 + q44 * n**2
    s66 = (q11 + q22 - 2 * q12) * m**2 * n**2 + q66 * (m**2 - n**2) ** 2
    return dict(s11=s11, s12=s12, s16=s16, s22=s22, s26=s26, s44=s44,
                s45=s45, s55=s55, s66=s66)


ABD_KEYS = ("a11", "a12", "a16", "a22", "a26", "a66", "a44", "a45", "a55",
            "b11", "b12", "b16", "b22", "b26", "b66",
            "d11", "d12", "d16", "d22", "d26", "d66", "m11", "I11")


def composite_plate_c(lh, rho, q11, q12, q22, q44, q55, q66, alpha, plies=None):
    """Laminate ABD, shear and mass terms from ply stiffnesses.

    Restates the undelaminated branch of
    ``flat_shell_engine/composite_plate_c_delam.m:47-87`` (identical to the
    integrals of ``composite_plate.m:52-83``).  ``plies`` restricts the sum to
    a subset of plies (the above/below-delamination branches ``:88-173``), the
    thickness h of the shear correction stays the full laminate's.
    """
    lay = len(lh)
    h, h1, h2 = ply_z(lh)
    rho = np.broadcast_to(np.asarray(rho, dtype=float), (lay,))
    s = rotated_q(q11, q12, q22, q44, q55, q66, alpha)
    s = {k: np.broadcast_to(v, (lay,)) for k, v in s.items()}
    out = {k: 0.0 for k in ABD_KEYS}
    for i in (range(lay) if plies is None else plies):
        d1 = h2[i] - h1[i]
        d2 = (h2[i] ** 2 - h1[i] ** 2) / 2
        d3 = (h2[i] ** 3 - h1[i] ** 3) / 3
        out["m11"] += rho[i] * (h2[i] - h1[i])
        out["I11"] += rho[i] * (h2[i] ** 3 - h1[i] ** 3) / 3
        shear = 5 / 4 * (h2[i] - h1[i] - 4 / 3 * (h2[i] ** 3 - h1[i] ** 3) / h**2)
        out["a44"] += s["s44"][i] * shear
        out["a45"] += s["s45"][i] * shear
        out["a55"] += s["s55"][i] * shear
        for kk in ("11", "12", "16", "22", "26", "66"):
            out["a" + kk] += s["s" + kk][i] * d1
            out["b" + kk] += s["s" + kk][i] * d2
            out["d" + kk] += s["s" + kk][i] * d3
    return out


def add_pzt_layer(abd, h, rho_pzt, pzt_thickness, Qpzt):
    """PZT layer on top of the laminate, ``composite_plate_c_delam_pzt.m:186-215``.

    Qpzt is the 6x6 elastic matrix in the reference's (x,y,z,xz?,yz?,xy)
    arrangement; indices below are the reference's 1-based ones minus one.
    """
    o = dict(abd)
    o["m11"] += rho_pzt * pzt_thickness
    o["I11"] += rho_pzt * ((h / 2 + pzt_thickness / 2) ** 3 - (h / 2) ** 3) / 3
    h2_ = h / 2 + pzt_thickness / 2
    h1_ = h / 2
    shear = 5 / 4 * (h2_ - h1_ - 4 / 3 * (h2_**3 - h1_**3) / (h + pzt_thickness) ** 2)
    o["a44"] += Qpzt[3, 3] * shear
    o["a45"] += Qpzt[3, 4] * shear
    o["a55"] += Qpzt[4, 4] * shear
    idx = {"11": (0, 0), "12": (0, 1), "16": (0, 5), "22": (1, 1), "26": (1, 5), "66": (5, 5)}
    for kk, (r, c) in idx.items():
        o["a" + kk] += Qpzt[r, c] * (h2_ - h1_)
        o["b" + kk] += Qpzt[r, c] * (h2_**2 - h1_**2) / 2
        o["d" + kk] += Qpzt[r, c] * (h2_**3 - h1_**3) / 3
    return o


def pzt_const(Spzt, dp, epsT, theta_deg):
    """``flat_shell_engine/pzt_const.m:3-37``."""
    th = theta_deg * np.pi / 180
    m = np.cos(th)
    n = np.sin(th)
    Tinv = np.array([[m**2, n**2, 0, 0, 0, -2 * m * n],
                     [n**2, m**2, 0, 0, 0, 2 * m * n],
                     [0, 0, 1, 0, 0, 0],
                     [0, 0, 0, m, n, 0],
                     [0, 0, 0, -n, m, 0],
                     [m * n, -m * n, 0, 0, 0, m**2 - n**2]])
    dp_ = Tinv @ np.asarray(dp).T
    ep = dp_.T @ np.linalg.inv(Spzt)
    gpzt = np.asarray(epsT, dtype=float)
    Qpzt = np.linalg.inv(Spzt)
    epzt = ep[:, [0, 1, 2, 5, 4, 3]]
    return dict(Qpzt=Qpzt, epzt=epzt, gpzt=gpzt, e31=ep[2, 0], e32=ep[2, 1], g33=epsT[2][2])


def engineering_2_c3d(e11, e22, e33, ni12, ni13, ni21, ni23, ni31, ni32, g12, g13, g23):
    """``src/models/common/engineering_2_C3D.m:26-40`` (Sierakowski eq. 2.33)."""
    Delta = (1 - ni12 * ni21 - ni13 * ni31 - ni12 * ni23 * ni31 - ni13 * ni21 * ni32 - ni23 * ni32)
    q11 = e11 * (1 - ni23 * ni32) / Delta
    q22 = e22 * (1 - ni31 * ni13) / Delta
    q33 = e33 * (1 - ni12 * ni21) / Delta
    q12 = (ni21 + ni31 * ni23) * e11 / Delta
    q13 = (ni31 + ni21 * ni32) * e11 / Delta
    q23 = (ni32 + ni12 * ni31) * e22 / Delta
    return np.array([[q11, q12, q13, 0, 0, 0],
                     [q12, q22, q23, 0, 0, 0],
                     [q13, q23, q33, 0, 0, 0],
                     [0, 0, 0, g23, 0, 0],
                     [0, 0, 0, 0, g13, 0],
                     [0, 0, 0, 0, 0, g12]])


def c3d_2_c2d(C):
    """``src/models/common/C3D_2_C2D.m:5-26`` (plane stress, eps_z = 0 shell)."""
    invC = np.linalg.inv(C)
    e11 = 1 / invC[0, 0]
    e22 = 1 / invC[1, 1]
    ni12 = -invC[1, 0] / invC[0, 0]
    ni21 = -invC[0, 1] / invC[1, 1]
    q11 = e11 / (1 - ni12 * ni21)
    q22 = e22 / (1 - ni12 * ni21)
    q12 = ni12 * e22 / (1 - ni12 * ni21)
    return q11, q12, q22, C[3, 3], C[4, 4], C[5, 5]


def damage_model(C, d):
    """``src/models/common/damage_model.m:19-46``: C_new = C - Cd(d)."""
    Cd11 = d * ((C[2, 2]) * (C[4, 4] / C[2, 2]) ** 2 - (C[4, 4] / C[2, 2]) ** 2)
    Cd22 = d * ((C[2, 2]) * (C[3, 3] / C[2, 2]) ** 2 - (C[3, 3] / C[2, 2]) ** 2)
    Cd33 = d * C[2, 2]
    Cd44 = d * C[3, 3]
    Cd55 = d * C[4, 4]
    Cd66 = d * (C[2, 2] * (C[3, 3] / C[2, 2]) * (C[4, 4] / C[2, 2]) - (C[3, 3] * C[4, 4] / C[2, 2] ** 2))
    Cd32 = d * C[2, 1]
    Cd31 = d * C[2, 0]
    Cd21 = (Cd22 - Cd66) / 2
    Cd = np.array([[Cd11, Cd21, Cd31, 0, 0, 0],
                   [Cd21, Cd22, Cd32, 0, 0, 0],
                   [Cd31, Cd32, Cd33, 0, 0, 0],
                   [0, 0, 0, Cd44, 0, 0],
                   [0, 0, 0, 0, Cd55, 0],
                   [0, 0, 0, 0, 0, Cd66]])
    return C - Cd


# --------------------------------------------------------------------------
# excitation, maps, mass
# --------------------------------------------------------------------------


def hanning_signal(dt, nft, f_1, f_2, t_1):
    """``flat_shell_engine/Hanning_signal.m:12-23``."""
    t_t = 1 / f_1
    t_2 = t_1 + t_t
    st = np.zeros(nft)
    t = np.zeros(nft)
    for nf in range(nft):
        t[nf] = nf * dt
        if t[nf] >= t_1 and t[nf] <= t_2:
            st[nf] = 0.5 * (1 - np.cos(2 * np.pi * f_1 * (t[nf] - t_2))) * np.sin(2 * np.pi * f_2 * (t[nf] - t_1))
    return t, st


def nodes_maps_fiborek(elementNodes1: np.ndarray, numberNodes: int, N: int, n_z: int = 1):
    """12-basket conflict-free scatter maps, ``flat_shell/mesher/nodesMaps_Fiborek.m:1-27``.

    elementNodes1 is 1-based [fen, npe].  Returns I_G, I_L as [rows, 12]
    1-based arrays (0 = empty slot), rows = npe*fen/12.  The per-node
    ``[~,S] = sort(H)`` is MATLAB's stable ascending sort.
    """
    n = N + 1
    npe = n * n * n_z
    fen = elementNodes1.shape[0]
    Psi = np.zeros(numberNodes + 1, dtype=np.int64)
    phi_E = np.zeros((numberNodes + 1, 12), dtype=np.int64)
    phi_L = np.zeros((numberNodes + 1, 12), dtype=np.int64)
    for e in range(1, fen + 1):
        for i in range(1, npe + 1):
            k = elementNodes1[e - 1, i - 1]
            Psi[k] += 1
            phi_E[k, Psi[k] - 1] = e
            phi_L[k, Psi[k] - 1] = i
    rows = npe * fen // 12
    I_G = np.zeros((rows, 12), dtype=np.int64)
    I_L = np.zeros((rows, 12), dtype=np.int64)
    H = np.zeros(12, dtype=np.int64)
    for k in range(1, numberNodes + 1):
        S = np.argsort(H, kind="stable")
        for i in range(Psi[k]):
            H[S[i]] += 1
            e = phi_E[k, i]
            I_G[H[S[i]] - 1, S[i]] = k
            I_L[H[S[i]] - 1, S[i]] = (e - 1) * npe + phi_L[k, i]
    return I_G, I_L


def basket_dofs(I_G, I_L, ndof_node: int = 5):
    """``mesher/global_local_12baskets_5dofs_v2.m:32-44`` (1-based, 0 stays 0)."""
    rows = I_G.shape[0]
    G = np.zeros((ndof_node * rows, 12), dtype=np.int64)
    L = np.zeros((ndof_node * rows, 12), dtype=np.int64)
    for d in range(ndof_node):
        G[d::ndof_node] = np.where(I_G > 0, ndof_node * I_G - (ndof_node - 1 - d), 0)
        L[d::ndof_node] = np.where(I_L > 0, ndof_node * I_L - (ndof_node - 1 - d), 0)
    return G, L


def basket_scatter(F2: np.ndarray, G: np.ndarray, L: np.ndarray, ndof: int):
    """12-basket assembly ``main_flat_shell.m:724-726`` (and mass ``:499-501``)."""
    F = np.zeros(ndof + 1)  # slot 0 absorbs empty basket slots
    F2p = np.concatenate(([0.0], F2))
    for b in range(12):
        g = G[:, b]
        F[g] = F[g] + F2p[L[:, b]]
    F[0] = 0.0
    return F[1:]


def mass_vector(WWDetJ, m11, I11, G, L, ndof):
    """Diagonal mass ``main_flat_shell.m:493-501`` (m11/I11 scalar or per local node)."""
    nl = WWDetJ.shape[0]
    mgL = np.zeros(5 * nl)
    mgL[0::5] = WWDetJ * m11
    mgL[1::5] = WWDetJ * I11
    mgL[2::5] = WWDetJ * m11
    mgL[3::5] = WWDetJ * I11
    mgL[4::5] = WWDetJ * m11
    return basket_scatter(mgL, G, L, ndof)


# --------------------------------------------------------------------------
# PZT actuator equivalent loads (main_flat_shell.m:144-225)
# --------------------------------------------------------------------------


def shape3d_prim(nx, ny, nz, Qx, Qy, Qz, x, y, z):
    """``src/models/common/shape3D_prim_v2.m``: derivatives of the nx*ny*nz
    shape functions (x fastest) at one point, |v| < 1e-12 -> 0."""
    ux = np.array([x ** j for j in range(nx)])
    uy = np.array([y ** j for j in range(ny)])
    uz = np.array([z ** j for j in range(nz)])
    Sx, Sy, Sz = ux @ Qx.T, uy @ Qy.T, uz @ Qz.T
    uxp = np.array([j * x ** (j - 1) if j else 0.0 for j in range(nx)])
    uyp = np.array([j * y ** (j - 1) if j else 0.0 for j in range(ny)])
    uzp = np.array([j * z ** (j - 1) if j else 0.0 for j in range(nz)])
    Sxp, Syp, Szp = Qx @ uxp, uyp @ Qy.T, uzp @ Qz.T
    n = nx * ny * nz
    Nx, Ny, Nz = np.zeros(n), np.zeros(n), np.zeros(n)
    cc = 0
    for j3 in range(nz):
        for j2 in range(ny):
            for j1 in range(nx):
                a = Sxp[j1] * Sy[j2] * Sz[j3]
                b = Sx[j1] * Syp[j2] * Sz[j3]
                c = Sx[j1] * Sy[j2] * Szp[j3]
                Nx[cc] = 0.0 if abs(a) < 1e-12 else a
                Ny[cc] = 0.0 if abs(b) < 1e-12 else b
                Nz[cc] = 0.0 if abs(c) < 1e-12 else c
                cc += 1
    return Nx, Ny, Nz


def coupl3d_global(epzt, gpzt, x, y, z, Qx, Qy, Qz, ksi, eta, dzeta, wx, wy, wz):
    """``flat_shell_engine/coupl3D_global.m:1-150``: piezo element matrices
    kufi [3N x N] and kfifi [N x N] of one 3D spectral element."""
    nx, ny, nz = len(ksi), len(eta), len(dzeta)
    N = nx * ny * nz
    kufi = np.zeros((3 * N, N))
    kfifi = np.zeros((N, N))
    for kz in range(nz):
        for ky in range(ny):
            for kx in range(nx):
                Px, Py, Pz = shape3d_prim(nx, ny, nz, Qx, Qy, Qz, ksi[kx], eta[ky], dzeta[kz])
                J = np.array([[Px @ x, Px @ y, Px @ z], [Py @ x, Py @ y, Py @ z], [Pz @ x, Pz @ y, Pz @ z]])
                Jj = J.reshape(-1)
                V3 = np.array([Jj[1] * Jj[5] - Jj[4] * Jj[2], Jj[3] * Jj[2] - Jj[0] * Jj[5], Jj[0] * Jj[4] - Jj[3] * Jj[1]])
                v3 = V3 / np.sqrt(V3 @ V3)
                v1 = Jj[:3] / np.sqrt(Jj[:3] @ Jj[:3])
                v2 = np.array([v3[1] * v1[2] - v3[2] * v1[1], -v3[0] * v1[2] + v3[2] * v1[0], v3[0] * v1[1] - v3[1] * v1[0]])
                v2 = v2 / np.sqrt(v2 @ v2)
                inJ = np.linalg.inv(J)
                detJ = np.linalg.det(J)
                w = wx[kx] * wy[ky] * wz[kz] * detJ
                Nxx = Px * inJ[0, 0] + Py * inJ[0, 1] + Pz * inJ[0, 2]
                Nyy = Px * inJ[1, 0] + Py * inJ[1, 1] + Pz * inJ[1, 2]
                Nzz = Px * inJ[2, 0] + Py * inJ[2, 1] + Pz * inJ[2, 2]
                B = np.zeros((6, 3 * N))
                B[0, 0::3] = Nxx
                B[1, 1::3] = Nyy
                B[2, 2::3] = Nzz
                B[3, 0::3] = Nyy
                B[3, 1::3] = Nxx
                B[4, 1::3] = Nzz
                B[4, 2::3] = Nyy
                B[5, 0::3] = Nzz
                B[5, 2::3] = Nxx
                Bfi = np.stack([Nxx * v1[0] + Nyy * v1[1] + Nzz * v1[2],
                                Nxx * v2[0] + Nyy * v2[1] + Nzz * v2[2],
                                Nxx * v3[0] + Nyy * v3[1] + Nzz * v3[2]])
                kufi += (B.T @ epzt.T @ Bfi) * w
                kfifi += Bfi.T @ gpzt @ Bfi * w
    return kufi, kfifi


def connect_pzt3d(nx, ny, nz, pztEl0, nodes1, coords, pzt_t, h):
    """``flat_shell/mesher/connect_pzt3D_to_plate_fun.m`` + ``remove_free_spec_nodes.m``:
    3D PZT elements on top of the plate elements pztEl0 (0-based); returns
    nodespzt [npzt, nx*ny*nz] 1-based (compact numbering), coordspzt and the
    plate node of each compact node (0 if not on the plate)."""
    ksi, _ = gll(nz)
    npzt = len(pztEl0)
    Nodemax = int(nodes1.max())
    nl = nx * ny
    nodespzt = np.zeros((npzt, nl * nz), dtype=np.int64)
    nodespzt[:, :nl] = nodes1[pztEl0, :nl]
    Bn, J = np.unique(nodespzt[:, :nl].T.reshape(-1), return_inverse=True)  # column-major as in MATLAB
    doflay = len(Bn)
    J = J.reshape(nl, npzt).T  # back to [element, node] order
    for k in range(1, nz):
        nodespzt[:, nl * k: nl * (k + 1)] = (np.arange(doflay) + 1 + Nodemax)[J]
        Nodemax += doflay
    coordspzt = np.zeros((Nodemax + 1, 3))
    for m in range(npzt):
        ne = pztEl0[m]
        for k in range(nz):
            idx = nodespzt[m, nl * k: nl * (k + 1)]
            coordspzt[idx, 0] = coords[nodes1[ne] - 1, 0]
            coordspzt[idx, 1] = coords[nodes1[ne] - 1, 1]
            coordspzt[idx, 2] = coords[nodes1[ne, :nl] - 1, 2] + (ksi[k] + 1) / 2 * pzt_t + h / 2
    used = np.unique(nodespzt)
    nodemap = np.zeros(Nodemax + 1, dtype=np.int64)
    nodemap[used] = np.arange(1, len(used) + 1)
    plate_of = np.where(used <= int(nodes1.max()), used, 0)
    return nodemap[nodespzt], coordspzt[used], plate_of


def find_boundary_nodes(nodes1, nx, ny):
    """``flat_shell/mesher/find_boundary_nodes.m``: nodes on the boundary of
    the element patch (corners shared by <= 2 elements, edge nodes of one
    element), in the reference's visiting order (1-based, may repeat)."""
    fen = nodes1.shape[0]
    mc = [0, nx - 1, nx * ny - nx, nx * ny - 1]
    e1 = list(range(1, nx - 1))
    e2 = [(k + 2) * nx - 1 for k in range(ny - 2)]
    e3 = list(range(nx * ny - nx + 1, nx * ny - 1))
    e4 = [(k + 1) * nx for k in range(ny - 2)]
    out = []
    for k in range(fen):
        others = [j for j in range(fen) if j != k]
        for i in range(4):
            cn = nodes1[k, mc[i]]
            nb = sum(1 for j in others for jc in range(4) if nodes1[j, mc[jc]] == cn)
            if nb <= 1:
                out.append(cn)
        for edge in (e1, e2, e3, e4):
            for i in edge:
                en = nodes1[k, i]
                nb = sum(1 for j in others for e in (e1, e2, e3, e4) for jc in e if nodes1[j, jc] == en)
                if nb == 0:
                    out.append(en)
    return np.array(out, dtype=np.int64)


def pzt_actuator_forces(nodes1, coords, pztEl0, pzt_t, h, V0, epzt, gpzt, nx=6, ny=6, nz=3):
    """Equivalent nodal loads Fa [5*nnode] of one PZT actuator driven at V0,
    ``main_flat_shell.m:144-225`` (bottom electrode 0 V, top V0, internal
    potential from the static condensation, in-plane forces of the bottom
    layer taken at the patch boundary, moments with lever h/2 + t/2)."""
    ksi, wx = gll(nx)
    eta, wy = gll(ny)
    dz, wz = gll(nz)
    Qx, Qy, Qz = vandermonde(ksi), vandermonde(eta), vandermonde(dz)
    nodespzt, cpzt, plate_of = connect_pzt3d(nx, ny, nz, pztEl0, nodes1, coords, pzt_t, h)
    nl = nx * ny
    EBC0 = np.unique(nodespzt[:, :nl])
    EBCI = np.unique(nodespzt[:, nl:-nl])
    EBCN = np.unique(nodespzt[:, -nl:])
    NofNodes = int(nodespzt.max())
    Kfiu = np.zeros((NofNodes, 3 * NofNodes))
    Kfifi = np.zeros((NofNodes, NofNodes))
    for c in range(len(pztEl0)):
        nd = nodespzt[c] - 1
        kufi, kfifi = coupl3d_global(epzt, gpzt, cpzt[nd, 0], cpzt[nd, 1], cpzt[nd, 2], Qx, Qy, Qz, ksi, eta, dz,
                                     wx, wy, wz)
        dof = (3 * nd[:, None] + np.arange(3)[None, :]).reshape(-1)
        Kfiu[np.ix_(nd, dof)] += kufi.T
        Kfifi[np.ix_(nd, nd)] += kfifi
    I, Nn = EBCI - 1, EBCN - 1
    Fetemp = Kfifi[np.ix_(I, Nn)] @ np.full(len(Nn), V0)
    fiAi = -np.linalg.solve(Kfifi[np.ix_(I, I)], Fetemp)
    FiA = np.zeros(NofNodes)
    FiA[Nn] = V0
    FiA[I] = fiAi
    FaL = Kfiu.T @ FiA
    bn_pzt = find_boundary_nodes(nodespzt[:, :nl], nx, ny)
    bn_glob = find_boundary_nodes(nodes1[pztEl0, :nl], nx, ny)
    nnode = coords.shape[0]
    FaxG = np.zeros(nnode)
    FayG = np.zeros(nnode)
    FaxG[bn_glob - 1] = FaL[0::3][bn_pzt - 1]
    FayG[bn_glob - 1] = FaL[1::3][bn_pzt - 1]
    Fa = np.zeros(5 * nnode)
    Fa[0::5] = FaxG
    Fa[2::5] = FayG
    Fa[1::5] = FaxG * (h / 2 + pzt_t / 2)
    Fa[3::5] = FayG * (h / 2 + pzt_t / 2)
    return Fa


# --------------------------------------------------------------------------
# 3D solid set-up (src/models/solid3D)
# --------------------------------------------------------------------------


def shape3d_blocks(nx=6, ny=6, nz=3):
    """Element blocks of Npx, Npy, Npz (main_spec3Dcuda_global_...:440-470 via
    shape3D_prim_v2.m evaluated at the GLL nodes, row = node c, x fastest)."""
    ksi, _ = gll(nx)
    eta, _ = gll(ny)
    dz, _ = gll(nz)
    Qx, Qy, Qz = vandermonde(ksi), vandermonde(eta), vandermonde(dz)
    n = nx * ny * nz
    Nx, Ny, Nz = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
    c = 0
    for kz in range(nz):
        for ky in range(ny):
            for kx in range(nx):
                Nx[c], Ny[c], Nz[c] = shape3d_prim(nx, ny, nz, Qx, Qy, Qz, ksi[kx], eta[ky], dz[kz])
                c += 1
    return Nx, Ny, Nz


def jacobians3d(nodes1, coords, Nx, Ny, Nz, nx=6, ny=6, nz=3):
    """J11 = Npx*X ... J33 = Npz*Z (:480-488); invJ = J^-1 of
    [[J11 J12 J13];[J21 J22 J23];[J31 J32 J33]] (inv_jacp.m is not in the
    reference tree; its use in strains_spec_p.m fixes it as the inverse);
    WWWDetJ = w_x w_y w_z det J (:600-619)."""
    X = coords[nodes1 - 1, 0]
    Y = coords[nodes1 - 1, 1]
    Z = coords[nodes1 - 1, 2]
    fen = nodes1.shape[0]
    J = np.zeros((fen, Nx.shape[0], 3, 3))
    for a, Np in enumerate((Nx, Ny, Nz)):
        J[:, :, 0, a] = X @ Np.T
        J[:, :, 1, a] = Y @ Np.T
        J[:, :, 2, a] = Z @ Np.T
    inv = np.linalg.inv(J)
    det = np.linalg.det(J)
    _, wx = gll(nx)
    _, wy = gll(ny)
    _, wz = gll(nz)
    www = np.einsum("k,j,i->kji", wz, wy, wx).reshape(-1)
    invJ = np.stack([inv[:, :, a, b].reshape(-1) for a in range(3) for b in range(3)])  # invJ_ab
    return invJ, (np.tile(www, fen) * det.reshape(-1))


def composite3d_ply(q11, q12, q13, q22, q23, q33, q44, q55, q66, alpha_deg):
    """Rotated ply constants, composite3D_transf_C.m:18-37, arranged as
    composite3D_transf.m:113-118 arranges them into D (D55 = s55, D56 = s45,
    D66 = s44).  Returns the 13 D entries of stresses_spec_p.m."""
    ar = alpha_deg * np.pi / 180
    m, n = np.cos(ar), np.sin(ar)
    if abs(m) < np.finfo(float).eps:
        m = 0.0
    if abs(n) < np.finfo(float).eps:
        n = 0.0
    s11 = q11 * m ** 4 + 2 * (q12 + 2 * q66) * m ** 2 * n ** 2 + q22 * n ** 4
    s12 = (q11 + q22 - 4 * q66) * m ** 2 * n ** 2 + q12 * (m ** 4 + n ** 4)
    s13 = q13 * m ** 2 + q23 * n ** 2
    s16 = (q11 - q12 - 2 * q66) * m ** 3 * n + (q12 - q22 + 2 * q66) * m * n ** 3
    s22 = q11 * n ** 4 + 2 * (q12 + 2 * q66) * m ** 2 * n ** 2 + q22 * m ** 4
    s23 = n ** 2 * q13 + m ** 2 * q23
    s33 = q33
    s26 = (q11 - q12 - 2 * q66) * n ** 3 * m + (q12 - q22 + 2 * q66) * n * m ** 3
    s36 = (q13 - q23) * m * n
    s44 = q44 * m ** 2 + q55 * n ** 2
    s45 = (q55 - q44) * m * n
    s55 = q55 * m ** 2 + q44 * n ** 2
    s66 = (q11 + q22 - 2 * q12 - 2 * q66) * m ** 2 * n ** 2 + q66 * (m ** 4 + n ** 4)
    return np.array([s11, s12, s13, s16, s22, s23, s26, s33, s36, s66, s55, s45, s44])


# --------------------------------------------------------------------------
# delamination topology
# --------------------------------------------------------------------------


def split_delam_nodes_flat_shell(nodes, coords, den1, nx, ny, boundary_nodes):
    """``src/models/flat_shell/mesher/split_delam_nodes_flat_shell.m:37-268``,
    literally: the per-element neighbour loops over corners and the four edge
    lists, the free-corner / boundary rule, then the split in ascending order
    of the inner node ids.  ``den1`` holds 1-based element numbers as in the
    reference; returns (nodes, coords, den_under, den_above), 1-based."""
    nodes = np.array(nodes, dtype=np.int64)
    coords = np.asarray(coords, dtype=float)
    den = [int(e) for e in den1]
    fen = nodes.shape[0]
    mc = [1, nx, nx * ny - nx + 1, nx * ny]
    edge1 = list(range(2, nx))
    edge2 = [(k + 1) * nx for k in range(1, ny - 1)]
    edge3 = list(range(nx * ny - nx + 2, nx * ny))
    edge4 = [k * nx + 1 for k in range(1, ny - 1)]
    den_under = list(den)
    den_above = [fen + k for k in range(1, len(den) + 1)]
    delamnodes = sorted(set(nodes[[e - 1 for e in den]].reshape(-1).tolist())) if den else []
    nodemax = int(nodes.max())
    nm = nodemax
    nodes = np.concatenate([nodes, nodes[[e - 1 for e in den]]]) if den else nodes

    def at(elem1, pos1):
        return int(nodes[elem1 - 1, pos1 - 1])

    outernodes, free_corner = [], []
    for k in range(len(den)):
        others = [j for j in range(len(den)) if j != k]
        for i in range(4):
            cn = at(den_above[k], mc[i])
            neighbours = 0
            for j in others:
                for jc in range(4):
                    if at(den_above[j], mc[jc]) == cn:
                        neighbours += 1
            if neighbours in (0, 1):
                outernodes.append(cn)
            if neighbours == 0:
                free_corner.append(cn)
        for edge in (edge1, edge2, edge3, edge4):
            for pos in edge:
                en = at(den_above[k], pos)
                neighbours = 0
                for j in others:
                    for lst in (edge1, edge2, edge3, edge4):
                        for jc in lst:
                            if at(den_above[j], jc) == en:
                                neighbours += 1
                if neighbours == 0:
                    outernodes.append(en)
    bset = set(int(b) for b in np.asarray(boundary_nodes).reshape(-1))
    special_corner = sorted(set(free_corner) & bset)
    if len(special_corner) == 3:
        special_corner = special_corner[1:3]
    outer = sorted(set(outernodes) - bset) + special_corner
    innernodes = sorted(set(delamnodes) - set(outer))
    for node in innernodes:
        nodemax += 1
        for i in range(len(den)):
            for j in range(nx * ny):
                if nodes[den_above[i] - 1, j] == node:
                    nodes[den_above[i] - 1, j] = nodemax
    coords_new = np.zeros((nodemax, 3))
    coords_new[:nm, :] = coords[:nm, :3]
    for a, u in zip(den_above, den_under):
        for j in range(nx * ny):
            coords_new[nodes[a - 1, j] - 1] = coords_new[nodes[u - 1, j] - 1]
    return nodes, coords_new, den_under, den_above


# --------------------------------------------------------------------------
# wavefield on a uniform grid
# --------------------------------------------------------------------------


def vandermonde2d(ksi, eta, nx, ny):
    """``src/models/solid3D/Vandermonde2D.m``: V(r,c) = ksi(i2)^(j2-1) eta(i1)^(j1-1),
    rows r over (eta point i1, ksi point i2), columns over (eta degree j1,
    ksi degree j2), ksi fastest; Q = inv(V)."""
    V = np.zeros((nx * ny, nx * ny))
    r = 0
    for i1 in range(ny):
        for i2 in range(nx):
            c = 0
            for j1 in range(ny):
                for j2 in range(nx):
                    V[r, c] = ksi[i2] ** j2 * eta[i1] ** j1
                    c += 1
            r += 1
    return np.linalg.inv(V)


def shape2dp(nx, ny, Q, x, y):
    """``src/models/solid3D/shape2Dp.m``: N = Q' f, f(c,:) = x^(j2-1) y^(j1-1)."""
    f = np.zeros((nx * ny, len(x)))
    c = 0
    for j1 in range(ny):
        for j2 in range(nx):
            f[c] = x ** j2 * y ** j1
            c += 1
    return Q.T @ f


def shape_derivatives2dp(nx, ny, Q, x, y):
    """``src/models/solid3D/shape_derivatives2Dp.m`` (0 * x^-1 terms kept as
    written: they are NaN at x = 0 exactly, as in MATLAB)."""
    fx = np.zeros((nx * ny, len(x)))
    fy = np.zeros((nx * ny, len(x)))
    c = 0
    with np.errstate(divide="ignore", invalid="ignore"):
        for j1 in range(ny):
            for j2 in range(nx):
                fx[c] = (j2 * x ** (j2 - 1.0)) * y ** j1
                fy[c] = x ** j2 * (j1 * y ** (j1 - 1.0))
                c += 1
    return Q.T @ fx, Q.T @ fy


def _colon(a, d, b):
    """MATLAB a:d:b as a + k*d, k = 0..floor((b-a)/d) (with a relative
    tolerance on the count, as MATLAB's colon)."""
    n = int(np.floor((b - a) / d + 1e-10)) + 1
    return a + np.arange(n) * d


def spec2meshgrid_flat_shell(nodes1, coords, Nx, Ny, fields, motion, shell_surface, h, den_under=(), den_above=(),
                             shape_order=5):
    """``src/models/flat_shell/flat_shell_engine/spec2meshgrid_flat_shell.m:55-583``.

    fields: dict of the frame vectors the motion needs, each [nFrames, nnode]
    ('x', 'Fix', 'y', 'Fiy', 'z' components of the chosen field_variable);
    den_under/den_above: 0-based element lists of one delamination (or empty).
    Returns (Data [Ny, Nx, nFrames] as the reference's, dict of set-up
    intermediates: xp, yp, owner (0-based), ksi_p, eta_p, max_err).
    The clamping at :268-271 comes after the shape functions are evaluated
    and has no effect; it is not restated.
    """
    Eps = 1e-8
    nodes1 = np.asarray(nodes1)
    coords = np.asarray(coords, float)
    n = shape_order + 1
    NofElNodes = n * n
    mc = np.array([1, n, n * n, n * n - n + 1]) - 1
    fen = nodes1.shape[0]
    if len(den_above):
        fen = fen - len(den_above)          # 'top' and 'bottom' remove as many elements
    ne = np.arange(fen)
    L = coords[:, 0].max() - coords[:, 0].min() - 2 * Eps
    xi = _colon(coords[:, 0].min() + Eps, L / (Nx - 1), coords[:, 0].max() - Eps)
    B = coords[:, 1].max() - coords[:, 1].min() - 2 * Eps
    yi = _colon(coords[:, 1].min() + Eps, B / (Ny - 1), coords[:, 1].max() - Eps)
    XI, YI = np.meshgrid(xi, yi)
    xp = XI.reshape(-1, order="F")
    yp = YI.reshape(-1, order="F")
    x = coords[nodes1[ne][:, mc] - 1, 0].T       # [4, fen]
    y = coords[nodes1[ne][:, mc] - 1, 1].T
    x21, x32, x43, x14 = x[1] - x[0], x[2] - x[1], x[3] - x[2], x[0] - x[3]
    y21, y32, y43, y14 = y[1] - y[0], y[2] - y[1], y[3] - y[2], y[0] - y[3]
    x1y21, y1x21 = x[0] * y21, y[0] * x21
    x2y32, y2x32 = x[1] * y32, y[1] * x32
    x3y43, y3x43 = x[2] * y43, y[2] * x43
    x4y14, y4x14 = x[3] * y14, y[3] * x14
    Pmin_x, Pmin_y, Pmax_x, Pmax_y = x.min(0), y.min(0), x.max(0), y.max(0)
    owner = np.zeros(len(xp), dtype=np.int64)
    for j in range(len(xp)):
        Ibb = np.nonzero((xp[j] >= Pmin_x) & (xp[j] <= Pmax_x) & (yp[j] >= Pmin_y) & (yp[j] <= Pmax_y))[0]
        if len(Ibb) == 1:
            owner[j] = Ibb[0]
        else:
            d1 = (xp[j] * y21[Ibb] - x1y21[Ibb]) - (yp[j] * x21[Ibb] - y1x21[Ibb])
            d2 = (xp[j] * y32[Ibb] - x2y32[Ibb]) - (yp[j] * x32[Ibb] - y2x32[Ibb])
            d3 = (xp[j] * y43[Ibb] - x3y43[Ibb]) - (yp[j] * x43[Ibb] - y3x43[Ibb])
            d4 = (xp[j] * y14[Ibb] - x4y14[Ibb]) - (yp[j] * x14[Ibb] - y4x14[Ibb])
            neg = (d1 < 0) & (d2 < 0) & (d3 < 0) & (d4 < 0)
            idx = np.nonzero(neg)[0]
            owner[j] = Ibb[0] if len(idx) == 0 else Ibb[idx[0]]
    ksi, _ = gll(n)
    eta, _ = gll(n)
    Ksi, Eta = np.meshgrid(ksi, eta)
    Ksi = Ksi.T.reshape(-1, order="F")            # reshape(Ksi',1,[])
    Eta = Eta.T.reshape(-1, order="F")
    en = nodes1[owner]                             # [npts, 36]
    x_0 = coords[en - 1, 0]
    y_0 = coords[en - 1, 1]
    point_no = np.argmin(np.sqrt((x_0 - xp[:, None]) ** 2 + (y_0 - yp[:, None]) ** 2), axis=1)
    r = np.arange(len(xp))
    x0, y0 = x_0[r, point_no], y_0[r, point_no]
    ksi0, eta0 = Ksi[point_no], Eta[point_no]
    # inverse Jacobian at the owner's first local node (<meshfile>_jacobians.mat)
    Q1 = vandermonde(ksi)
    Nprimx, Nprimy = shape2d_prim(n, n, Q1, Q1, ksi, eta)
    jac = jacobians(nodes1, coords, Nprimx, Nprimy)
    n1 = owner * NofElNodes
    ksi_p = ksi0 + jac["invJ11"][n1] * (xp - x0) + jac["invJ12"][n1] * (yp - y0)
    eta_p = eta0 + jac["invJ21"][n1] * (xp - x0) + jac["invJ22"][n1] * (yp - y0)
    Q = vandermonde2d(ksi, eta, n, n)
    N = shape2dp(n, n, Q, ksi_p, eta_p)            # [36, npts]
    xe = x_0.T                                     # [36, npts]
    ye = y_0.T
    x1 = np.einsum("kp,kp->p", N, xe)
    y1 = np.einsum("kp,kp->p", N, ye)
    for _ in range(3):
        ksi0, eta0, x0, y0 = ksi_p, eta_p, x1, y1
        Npx, Npy = shape_derivatives2dp(n, n, Q, ksi0, eta0)
        J11 = np.einsum("kp,kp->p", Npx, xe)
        J12 = np.einsum("kp,kp->p", Npy, xe)
        J21 = np.einsum("kp,kp->p", Npx, ye)
        J22 = np.einsum("kp,kp->p", Npy, ye)
        a = 1.0 / (J11 * J22 - J12 * J21)
        ksi_p = ksi0 + (a * J22) * (xp - x0) + (a * (-J12)) * (yp - y0)
        eta_p = eta0 + (a * (-J21)) * (xp - x0) + (a * J11) * (yp - y0)
        N = shape2dp(n, n, Q, ksi_p, eta_p)
        x1 = np.einsum("kp,kp->p", N, xe)
        y1 = np.einsum("kp,kp->p", N, ye)
    max_err = float(np.max(np.sqrt((xp - x1) ** 2 + (yp - y1) ** 2)))
    # motion values per frame (:281-510)
    s = h / 2 if shell_surface == "top" else -h / 2
    F = {k: np.atleast_2d(np.asarray(v, float)) for k, v in fields.items()}
    if motion == 1:
        U = F["x"]
    elif motion == 2:
        U = F["y"]
    elif motion == 3:
        U = F["z"]
    elif motion == 4:
        U = F["Fix"]
    elif motion == 5:
        U = F["Fiy"]
    elif motion == 6:
        U = F["x"] + s * F["Fix"]
    elif motion == 7:
        U = F["y"] + s * F["Fiy"]
    elif motion == 8:
        U = np.sqrt((F["x"] + s * F["Fix"]) ** 2 + (F["y"] + s * F["Fiy"]) ** 2)
    else:
        U = np.sqrt((F["x"] + s * F["Fix"]) ** 2 + (F["y"] + s * F["Fiy"]) ** 2 + F["z"] ** 2)
    U = U.copy()
    if shell_surface == "top" and len(den_above):
        nu = nodes1[np.asarray(den_under)].reshape(-1, order="F") - 1
        na = nodes1[np.asarray(den_above)].reshape(-1, order="F") - 1
        U[:, nu] = U[:, na]
    if Nx != Ny:
        raise ValueError("the reference stores reshape(ZI, Nx, Ny) into Data(Ny, Nx, :): Nx must equal Ny")
    Data = np.zeros((Ny, Nx, U.shape[0]))
    for f in range(U.shape[0]):
        ZA = U[f][en - 1].T                         # [36, npts]
        ZI = np.einsum("kp,kp->p", N, ZA)
        Data[:, :, f] = ZI.reshape((Nx, Ny), order="F")
    return Data, dict(xp=xp, yp=yp, owner=owner, ksi_p=ksi_p, eta_p=eta_p, max_err=max_err)


# --------------------------------------------------------------------------
# quad mesh to spectral elements
# --------------------------------------------------------------------------


def change_turn_quad(nodes, pqs):
    """``src/models/flat_shell/mesher/change_turn_quad.m``: 2x2 Lagrange
    derivatives at the corners (tensor order m = [1,2,4,3]); an element with a
    non-positive Jacobian determinant is renumbered m3 = [1,4,3,2]."""
    nodes = np.array(nodes, dtype=np.int64)
    n = 2
    m = [0, 1, 3, 2]
    m3 = [0, 3, 2, 1]
    ksi = np.array([-1.0, 1.0])
    V = np.array([[ksi[j] ** i for j in range(n)] for i in range(n)])
    Q = np.linalg.inv(V)
    Vx = np.zeros((n, n))
    for k in range(n):
        for i in range(n):
            for j in range(1, n):
                Vx[k, i] += Q[i, j] * j * ksi[k] ** (j - 1)
    for ne in range(nodes.shape[0]):
        x = [pqs[nodes[ne, m[c]] - 1, 0] for c in range(4)]
        y = [pqs[nodes[ne, m[c]] - 1, 1] for c in range(4)]
        bad = False
        for j in range(n):
            for i in range(n):
                J11 = sum(Vx[i, kx] * x[j * n + kx] for kx in range(n))
                J12 = sum(Vx[i, kx] * y[j * n + kx] for kx in range(n))
                J22 = sum(Vx[j, ky] * y[ky * n + i] for ky in range(n))
                J21 = sum(Vx[j, ky] * x[ky * n + i] for ky in range(n))
                if J11 * J22 - J12 * J21 <= 0:
                    bad = True
        if bad:
            nodes[ne] = nodes[ne, m3]
    return nodes


def quad2spectral_fiborek(elementNodes_fem, nodeCoordinates_fem, N):
    """``src/models/flat_shell/mesher/quad2spectral_Fiborek.m``, step by step:
    rounded edge midpoints (``edgegeometry``), edge-interior nodes numbered by
    ``unique(...,'rows')``, interior nodes as intersections of the lines between
    opposite edge nodes (Cramer's rule of the sparse block products, taken in
    the column-major order of ``W(AA)``), the row assembly ``elementNodes_pl3``
    and the boundary nodes of edges whose midpoint occurs once.  1-based."""
    efem = np.asarray(elementNodes_fem, dtype=np.int64)
    pos = np.asarray(nodeCoordinates_fem, dtype=float)
    n = N + 1
    fen = efem.shape[0]
    n_int = n - 2
    ksi, _ = gll(n)
    ksi_int = ksi[1:n - 1]

    def mround(v):
        return np.sign(v) * np.floor(np.abs(v) + 0.5)

    def edgegeometry(dim):
        nC = pos[efem[:, [0, 1, 2, 3, 0]] - 1, dim]                 # [fen, 5]
        mid = (nC[:, 1:5] + nC[:, 0:4]) / 2
        mid = mround(mid.reshape(-1) * 1e6) * 1e-6                   # reshape(mid',[],1)
        ln = ((nC[:, 1:5] - nC[:, 0:4]) / 2).reshape(-1)
        return mid, ln

    mids, lens, temps = [], [], []
    for dim in range(3):
        mid, ln = edgegeometry(dim)
        mids.append(mid)
        lens.append(ln)
        temps.append((mid[:, None] + ln[:, None] * ksi_int[None, :]).reshape(-1))   # reshape(tmp',[],1)
    ic = np.stack(temps, axis=1)
    b1, n1 = np.unique(ic, axis=0, return_inverse=True)          # unique(...,'first','rows')
    n1 = n1.reshape(-1) + 1
    nce = b1
    en_edge = n1.reshape(fen, 4 * n_int)
    maxe = int(en_edge.max())
    en_int = (np.arange(1, fen * n_int ** 2 + 1) + maxe).reshape(fen, n_int ** 2)
    cols = lambda lo, hi, step=1: np.arange(lo, hi + (1 if step > 0 else -1), step) - 1
    n_el1 = en_edge[:, cols(1, n_int)]
    n_el2 = en_edge[:, cols(1 + n_int, 2 * n_int)]
    n_el3 = en_edge[:, cols(3 * n_int, 1 + 2 * n_int, -1)]
    n_el4 = en_edge[:, cols(4 * n_int, 1 + 3 * n_int, -1)]
    X_int, Y_int = [], []
    for e in range(fen):
        x1, y1 = nce[n_el1[e] - 1, 0], nce[n_el1[e] - 1, 1]
        x3, y3 = nce[n_el3[e] - 1, 0], nce[n_el3[e] - 1, 1]
        x2, y2 = nce[n_el2[e] - 1, 0], nce[n_el2[e] - 1, 1]
        x4, y4 = nce[n_el4[e] - 1, 0], nce[n_el4[e] - 1, 1]
        A13, B13, C13 = y3 - y1, x1 - x3, (y1 - y3) * x1 + (x3 - x1) * y1
        A42, B42, C42 = y2 - y4, x4 - x2, (y4 - y2) * x4 + (x2 - x4) * y4
        for mm in range(n_int):          # column of the block (42 index)
            for kk in range(n_int):      # row of the block (13 index)
                W = A13[kk] * B42[mm] - B13[kk] * A42[mm]
                X_int.append((B13[kk] * C42[mm] - C13[kk] * B42[mm]) / W)
                Y_int.append((C13[kk] * A42[mm] - A13[kk] * C42[mm]) / W)
    zs = np.unique(nce[:, 2])
    nci = np.stack([np.array(X_int), np.array(Y_int), np.full(len(X_int), zs[0])], axis=1)
    en_int_all = np.concatenate([en_edge, en_int], axis=1) + int(efem.max())
    ensem = np.concatenate([efem, en_int_all], axis=1)            # columns 1..4, then 4 + ...
    spec_coords = np.concatenate([pos, nce, nci])
    pl3 = np.zeros_like(ensem)
    for ii in range(1, n + 1):
        if ii == 1:
            c = [1] + list(range(4 + 1, 4 + n_int + 1)) + [2]
        elif ii < n:
            c = ([4 + 4 * n_int - ii + 2] + list(range((ii - 2) * n_int + 1 + 4 + 4 * n_int,
                                                       (ii - 2) * n_int + 4 + 4 * n_int + n_int + 1))
                 + [ii - 1 + 4 + 1 * n_int])
        else:
            c = [4] + list(range(4 + 3 * n_int, 4 + 2 * n_int, -1)) + [3]
        pl3[:, n * (ii - 1):n * ii] = ensem[:, np.array(c) - 1]
    mid3 = np.stack(mids, axis=1)
    _, n0, cnt = np.unique(mid3, axis=0, return_inverse=True, return_counts=True)
    n0 = n0.reshape(-1)
    single = cnt[n0] == 1
    edges = [list(range(1, n + 1)), list(range(n, n * n + 1, n)), list(range(1 + n * (n - 1), n * n + 1)),
             list(range(1, 1 + n * (n - 1) + 1, n))]
    en_edge_cols = pl3[:, np.array(sum(edges, [])) - 1]           # [fen, 4n]
    mask = np.repeat(single.reshape(fen, 4), n, axis=1)
    boundary = np.unique(en_edge_cols[mask])
    return pl3, spec_coords, boundary
