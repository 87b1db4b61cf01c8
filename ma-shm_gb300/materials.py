"""Laminate, piezoelectric and damage material models (host set-up, FP64).

Produces the per-material rows of the engine's material table
(SHM_MAT_STRIDE = 23 values: a11 a12 a16 a22 a26 a66 a44 a45 a55 b11 b12 b16
b22 b26 b66 d11 d12 d16 d22 d26 d66 m11 I11), i.e. what the reference's
composite_plate*.m functions return (src/models/flat_shell/flat_shell_engine/
composite_plate.m:33-83, composite_plate_c_delam.m:47-173,
composite_plate_c_delam_pzt.m:175-217).  The ply rotation is written as the
matrix product Qbar = Ts^-1 Q Te of the stress/strain transformation matrices
rather than the expanded formulas; both give the same numbers (tests compare).
"""
from __future__ import annotations

import numpy as np

ABD_KEYS = ("a11", "a12", "a16", "a22", "a26", "a66", "a44", "a45", "a55",
            "b11", "b12", "b16", "b22", "b26", "b66",
            "d11", "d12", "d16", "d22", "d26", "d66", "m11", "I11")


def ply_stiffness(E11, E22, nu12, G12, G13, G23):
    """Plane-stress reduced stiffness q11 q12 q22 q44 q55 q66 of a ply
    (composite_plate.m:23-28; q44 = G23, q55 = G13, q66 = G12)."""
    nu21 = E22 / E11 * nu12
    d = 1.0 - nu12 * nu21
    return dict(q11=E11 / d, q12=nu12 * E22 / d, q22=E22 / d, q44=G23, q55=G13, q66=G12)


def rotated_ply(q, angle_deg):
    """In-plane Qbar (3x3, engineering shear) and transverse Qs (2x2, order yz, xz)."""
    t = np.deg2rad(angle_deg)
    m, n = np.cos(t), np.sin(t)
    Q = np.array([[q["q11"], q["q12"], 0.0], [q["q12"], q["q22"], 0.0], [0.0, 0.0, q["q66"]]])
    Ts = np.array([[m * m, n * n, 2 * m * n], [n * n, m * m, -2 * m * n], [-m * n, m * n, m * m - n * n]])
    Te = np.array([[m * m, n * n, m * n], [n * n, m * m, -m * n], [-2 * m * n, 2 * m * n, m * m - n * n]])
    Qbar = np.linalg.solve(Ts, Q @ Te)
    R = np.array([[m, n], [-n, m]])
    Qs = R @ np.diag([q["q44"], q["q55"]]) @ R.T
    return Qbar, Qs


def laminate(q, rho, ply_t, angles, plies=None) -> dict:
    """A, B, D, shear (5/4 parabolic weighting) and mass terms of a laminate.

    Plies are listed from the top surface (z = +h/2) downward as in the
    reference (lay_const.m:16-21); ``plies`` limits the integrals to a subset
    (sub-laminates above/below a delamination) while keeping the mid-plane and
    the shear-correction thickness of the full laminate.
    """
    ply_t = np.asarray(ply_t, dtype=float)
    angles = np.asarray(angles, dtype=float)
    rho = np.broadcast_to(np.asarray(rho, dtype=float), ply_t.shape)
    h = float(ply_t.sum())
    ztop = h / 2 - np.concatenate(([0.0], np.cumsum(ply_t)[:-1]))
    zbot = ztop - ply_t
    A = np.zeros((3, 3)); B = np.zeros((3, 3)); D = np.zeros((3, 3)); S = np.zeros((2, 2))
    m11 = I11 = 0.0
    idx = range(len(ply_t)) if plies is None else plies
    for i in idx:
        Qbar, Qs = rotated_ply(q, angles[i])
        z1, z2 = zbot[i], ztop[i]
        A += Qbar * (z2 - z1)
        B += Qbar * (z2 ** 2 - z1 ** 2) / 2
        D += Qbar * (z2 ** 3 - z1 ** 3) / 3
        S += Qs * 1.25 * ((z2 - z1) - 4.0 / 3.0 * (z2 ** 3 - z1 ** 3) / h ** 2)
        m11 += rho[i] * (z2 - z1)
        I11 += rho[i] * (z2 ** 3 - z1 ** 3) / 3
    out = {}
    for name, M in (("a", A), ("b", B), ("d", D)):
        out[name + "11"], out[name + "12"], out[name + "16"] = M[0, 0], M[0, 1], M[0, 2]
        out[name + "22"], out[name + "26"], out[name + "66"] = M[1, 1], M[1, 2], M[2, 2]
    out["a44"], out["a45"], out["a55"] = S[0, 0], S[0, 1], S[1, 1]
    out["m11"], out["I11"] = m11, I11
    out["h"] = h
    return out


def table_row(lam: dict) -> np.ndarray:
    return np.array([lam[k] for k in ABD_KEYS], dtype=float)


def pzt_material(S, d, epsT, theta_deg=0.0):
    """Piezo stiffness and stress constants from compliance S (6x6, order
    x y z yz xz xy), charge constants d (3x6) and permittivity epsT (3x3),
    restating pzt_const.m:3-37: C = S^-1, e = d_rot C, e31, e32, g33 = epsT33."""
    t = np.deg2rad(theta_deg)
    m, n = np.cos(t), np.sin(t)
    # strain-vector transformation for a rotation about z (Voigt x y z yz xz xy)
    R = np.array([[m * m, n * n, 0, 0, 0, -2 * m * n],
                  [n * n, m * m, 0, 0, 0, 2 * m * n],
                  [0, 0, 1, 0, 0, 0],
                  [0, 0, 0, m, n, 0],
                  [0, 0, 0, -n, m, 0],
                  [m * n, -m * n, 0, 0, 0, m * m - n * n]])
    drot = (R @ np.asarray(d, float).T).T
    Cp = np.linalg.inv(np.asarray(S, float))
    e = drot @ Cp
    return dict(Qpzt=Cp, e=e, epzt=e[:, [0, 1, 2, 5, 4, 3]], gpzt=np.asarray(epsT, float),
                e31=e[2, 0], e32=e[2, 1], g33=float(np.asarray(epsT)[2, 2]))


def add_piezo_layer(lam: dict, Qpzt: np.ndarray, rho_pzt: float, t_pzt: float) -> dict:
    """Surface-bonded PZT layer between z = h/2 and h/2 + t/2 added to a laminate
    row, the reference's treatment (composite_plate_c_delam_pzt.m:186-215,
    including its lever arm t/2 and shear thickness h + t)."""
    return add_surface_layer(lam, Qpzt, rho_pzt, t_pzt)


def add_added_mass(lam: dict, Qm: np.ndarray, rho_m: float, t_m: float) -> dict:
    """Added mass bonded to the top surface (composite_plate_c_added_mass_pzt.m:195-240):
    the same surface-layer integrals as the PZT layer with the mass's own
    stiffness Qm (6x6, Voigt x y z yz xz xy), density and thickness."""
    return add_surface_layer(lam, Qm, rho_m, t_m)


def add_surface_layer(lam: dict, Qpzt: np.ndarray, rho_pzt: float, t_pzt: float) -> dict:
    """Layer between z = h/2 and h/2 + t/2 on a laminate row (lever arm t/2,
    shear-correction thickness h + t, as the reference's surface layers)."""
    h = lam["h"]
    o = dict(lam)
    z1, z2 = h / 2, h / 2 + t_pzt / 2
    o["m11"] += rho_pzt * t_pzt
    o["I11"] += rho_pzt * (z2 ** 3 - z1 ** 3) / 3
    shear = 1.25 * ((z2 - z1) - 4.0 / 3.0 * (z2 ** 3 - z1 ** 3) / (h + t_pzt) ** 2)
    o["a44"] += Qpzt[3, 3] * shear
    o["a45"] += Qpzt[3, 4] * shear
    o["a55"] += Qpzt[4, 4] * shear
    pos = {"11": (0, 0), "12": (0, 1), "16": (0, 5), "22": (1, 1), "26": (1, 5), "66": (5, 5)}
    for k, (r, c) in pos.items():
        o["a" + k] += Qpzt[r, c] * (z2 - z1)
        o["b" + k] += Qpzt[r, c] * (z2 ** 2 - z1 ** 2) / 2
        o["d" + k] += Qpzt[r, c] * (z2 ** 3 - z1 ** 3) / 3
    return o


def orthotropic_c3d(E11, E22, E33, nu12, nu13, nu23, G12, G13, G23):
    """3D stiffness (Voigt x y z yz xz xy) of an orthotropic ply: inverse of the
    compliance matrix (engineering_2_C3D.m gives the same closed form)."""
    S = np.zeros((6, 6))
    S[0, 0], S[1, 1], S[2, 2] = 1 / E11, 1 / E22, 1 / E33
    S[0, 1] = S[1, 0] = -nu12 / E11
    S[0, 2] = S[2, 0] = -nu13 / E11
    S[1, 2] = S[2, 1] = -nu23 / E22
    S[3, 3], S[4, 4], S[5, 5] = 1 / G23, 1 / G13, 1 / G12
    return np.linalg.inv(S)


def c3d_to_plate(C):
    """Plane-stress plate constants from a 3D stiffness (C3D_2_C2D.m)."""
    S = np.linalg.inv(C)
    E1, E2 = 1 / S[0, 0], 1 / S[1, 1]
    nu12 = -S[1, 0] / S[0, 0]
    nu21 = -S[0, 1] / S[1, 1]
    d = 1 - nu12 * nu21
    return dict(q11=E1 / d, q12=nu12 * E2 / d, q22=E2 / d, q44=C[3, 3], q55=C[4, 4], q66=C[5, 5])


def degrade_c3d(C, d):
    """Delamination-type degradation C - Cd(d) of a 3D stiffness
    (src/models/common/damage_model.m:19-46)."""
    c33, c44, c55 = C[2, 2], C[3, 3], C[4, 4]
    r5, r4 = c55 / c33, c44 / c33
    Cd = np.zeros((6, 6))
    Cd[0, 0] = d * (c33 * r5 ** 2 - r5 ** 2)
    Cd[1, 1] = d * (c33 * r4 ** 2 - r4 ** 2)
    Cd[2, 2] = d * c33
    Cd[3, 3] = d * c44
    Cd[4, 4] = d * c55
    Cd[5, 5] = d * (c33 * r4 * r5 - c44 * c55 / c33 ** 2)
    Cd[2, 1] = Cd[1, 2] = d * C[2, 1]
    Cd[2, 0] = Cd[0, 2] = d * C[2, 0]
    Cd[1, 0] = Cd[0, 1] = (Cd[1, 1] - Cd[5, 5]) / 2
    return C - Cd


# The laminate of the synthetic plates: quasi-isotropic CFRP [0/90/45/-45]s,
# 8 plies of 0.4875 mm (3.9 mm), E11 130, E22 10, G12 = G13 5, G23 3.5 GPa,
# nu12 0.3, rho 1570 kg/m^3.
CFRP_PLY = dict(E11=130e9, E22=10e9, nu12=0.3, G12=5e9, G13=5e9, G23=3.5e9)
CFRP_RHO = 1570.0
CFRP_ANGLES = (0.0, 90.0, 45.0, -45.0, -45.0, 45.0, 90.0, 0.0)
CFRP_PLY_T = (0.4875e-3,) * 8


def cfrp_laminate() -> dict:
    q = ply_stiffness(**CFRP_PLY)
    return laminate(q, CFRP_RHO, CFRP_PLY_T, CFRP_ANGLES)


# PZT-5A-like disc: compliance at constant field, d constants, permittivity.
def pzt5a():
    E11, E33, nu = 61e9, 53.2e9, 0.35
    S = np.zeros((6, 6))
    S[0, 0] = S[1, 1] = 1 / E11
    S[2, 2] = 1 / E33
    S[0, 1] = S[1, 0] = -nu / E11
    S[0, 2] = S[2, 0] = S[1, 2] = S[2, 1] = -nu / E33
    S[3, 3] = S[4, 4] = 1 / 21.1e9
    S[5, 5] = 2 * (1 + nu) / E11
    d = np.zeros((3, 6))
    d[0, 4] = d[1, 3] = 584e-12
    d[2, 0] = d[2, 1] = -171e-12
    d[2, 2] = 374e-12
    eps0 = 8.854e-12
    epsT = np.diag([1730 * eps0, 1730 * eps0, 1700 * eps0])
    return dict(S=S, d=d, epsT=epsT, rho=7750.0)


def ply_c3d_rotated(C: np.ndarray, angle_deg: float) -> np.ndarray:
    """3D ply stiffness (Voigt x y z yz xz xy) rotated about z by the ply angle:
    Cbar = T^-1 C T^-T with the stress transformation T (Bond matrix)."""
    t = np.deg2rad(angle_deg)
    m, n = np.cos(t), np.sin(t)
    T = np.array([[m * m, n * n, 0, 0, 0, 2 * m * n],
                  [n * n, m * m, 0, 0, 0, -2 * m * n],
                  [0, 0, 1, 0, 0, 0],
                  [0, 0, 0, m, -n, 0],
                  [0, 0, 0, n, m, 0],
                  [-m * n, m * n, 0, 0, 0, m * m - n * n]])
    Ti = np.linalg.inv(T)
    return Ti @ C @ Ti.T


def solid_row(C: np.ndarray, rho: float, shear_as_reference: bool = True) -> np.ndarray:
    """Material row of the 3D solid (D11 D12 D13 D14 D22 D23 D24 D33 D34 D44 D55
    D56 D66 rho, strain order xx yy zz xy yz xz) from a stiffness in the order
    x y z yz xz xy.  With ``shear_as_reference`` the two transverse shear terms
    are placed as the reference's composite3D_transf.m:107-108 places them
    (D55 from the xz term, D66 from the yz term); otherwise D55 = C_yz,yz."""
    xy, yz, xz = 5, 3, 4
    D = dict(D11=C[0, 0], D12=C[0, 1], D13=C[0, 2], D14=C[0, xy], D22=C[1, 1], D23=C[1, 2], D24=C[1, xy],
             D33=C[2, 2], D34=C[2, xy], D44=C[xy, xy])
    if shear_as_reference:
        D55, D56, D66 = C[xz, xz], C[yz, xz], C[yz, yz]
    else:
        D55, D56, D66 = C[yz, yz], C[yz, xz], C[xz, xz]
    return np.array([D["D11"], D["D12"], D["D13"], D["D14"], D["D22"], D["D23"], D["D24"], D["D33"], D["D34"],
                     D["D44"], D55, D56, D66, rho], float)


def cfrp_c3d() -> np.ndarray:
    """3D stiffness of the synthetic CFRP ply (E33 = E22, nu13 = nu12, nu23
    from G23 = E22 / (2 (1 + nu23)))."""
    p = CFRP_PLY
    nu23 = p["E22"] / (2 * p["G23"]) - 1.0
    return orthotropic_c3d(p["E11"], p["E22"], p["E22"], p["nu12"], p["nu12"], nu23, p["G12"], p["G13"], p["G23"])
