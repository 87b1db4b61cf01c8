"""Dense element matrices of the flat-shell spectral element (host, FP64).

Used for the stable time step (largest generalized eigenvalue of the lumped
element pair, an upper bound of the assembled system's, so dt = safety *
2/sqrt(lambda_max) is stable for the central-difference scheme) and by the
tests as an independent B^T C B derivation of the operator that the kernels
apply matrix-free.

DOF order per node: u, phi_x, v, phi_y, w (main_flat_shell.m:432-436);
generalised strains: eps_x, eps_y, gamma_xy, kappa_x, kappa_y, kappa_xy,
gamma_yz = phi_y + w_y, gamma_xz = phi_x + w_x (main_flat_shell.m:674-681).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from .mesh import gll_points


def gll_derivative_matrix(n: int):
    x, w = gll_points(n)
    lam = np.array([1.0 / np.prod([x[j] - x[k] for k in range(n) if k != j]) for j in range(n)])
    D = np.zeros((n, n))
    for r in range(n):
        for c in range(n):
            if c != r:
                D[r, c] = (lam[c] / lam[r]) / (x[r] - x[c])
        D[r, r] = -D[r].sum()
    D[np.abs(D) < 1e-12] = 0.0
    return x, w, D


def constitutive(lam: dict) -> np.ndarray:
    """8x8 [N; M; Q] = C [eps; kappa; gamma_s]."""
    A = np.array([[lam["a11"], lam["a12"], lam["a16"]], [lam["a12"], lam["a22"], lam["a26"]],
                  [lam["a16"], lam["a26"], lam["a66"]]])
    B = np.array([[lam["b11"], lam["b12"], lam["b16"]], [lam["b12"], lam["b22"], lam["b26"]],
                  [lam["b16"], lam["b26"], lam["b66"]]])
    D = np.array([[lam["d11"], lam["d12"], lam["d16"]], [lam["d12"], lam["d22"], lam["d26"]],
                  [lam["d16"], lam["d26"], lam["d66"]]])
    S = np.array([[lam["a44"], lam["a45"]], [lam["a45"], lam["a55"]]])
    Cm = np.zeros((8, 8))
    Cm[:3, :3], Cm[:3, 3:6], Cm[3:6, :3], Cm[3:6, 3:6], Cm[6:, 6:] = A, B, B, D, S
    return Cm


def element_stiffness(xy: np.ndarray, lam: dict, order: int = 5) -> np.ndarray:
    """K_e (5*36 square) of a straight-sided or curved quad with nodes xy [36,2]
    (local order xi fastest), collocated GLL quadrature."""
    n = order + 1
    _, w, D = gll_derivative_matrix(n)
    X = xy[:, 0].reshape(n, n)   # [k (eta), i (xi)]
    Y = xy[:, 1].reshape(n, n)
    J11 = X @ D.T   # dx/dxi at (k,i)
    J21 = Y @ D.T
    J12 = D @ X     # dx/deta
    J22 = D @ Y
    det = J11 * J22 - J12 * J21
    i11, i12, i21, i22 = J22 / det, -J12 / det, -J21 / det, J11 / det
    Cm = constitutive(lam)
    nd = n * n
    K = np.zeros((5 * nd, 5 * nd))
    for k in range(n):
        for i in range(n):
            # d/dxi and d/deta of nodal shape functions at node (i, k)
            dxi = np.zeros(nd)
            deta = np.zeros(nd)
            dxi[k * n: k * n + n] = D[i]
            deta[np.arange(n) * n + i] = D[k]
            ddx = dxi * i11[k, i] + deta * i21[k, i]
            ddy = dxi * i12[k, i] + deta * i22[k, i]
            Bm = np.zeros((8, 5 * nd))
            u, fx, v, fy, wz = (slice(f, 5 * nd, 5) for f in range(5))
            Bm[0, u] = ddx
            Bm[1, v] = ddy
            Bm[2, u] = ddy
            Bm[2, v] = ddx
            Bm[3, fx] = ddx
            Bm[4, fy] = ddy
            Bm[5, fx] = ddy
            Bm[5, fy] = ddx
            c = k * n + i
            Bm[6, 5 * c + 3] += 1.0   # phi_y
            Bm[6, wz] += ddy
            Bm[7, 5 * c + 1] += 1.0   # phi_x
            Bm[7, wz] += ddx
            K += (w[i] * w[k] * det[k, i]) * (Bm.T @ Cm @ Bm)
    return K


def element_mass(xy: np.ndarray, lam: dict, order: int = 5) -> np.ndarray:
    n = order + 1
    _, w, D = gll_derivative_matrix(n)
    X = xy[:, 0].reshape(n, n)
    Y = xy[:, 1].reshape(n, n)
    det = (X @ D.T) * (D @ Y) - (D @ X) * (Y @ D.T)
    W = (w[None, :] * w[:, None] * det).reshape(-1)
    m = np.zeros(5 * n * n)
    m[0::5] = W * lam["m11"]
    m[1::5] = W * lam["I11"]
    m[2::5] = W * lam["m11"]
    m[3::5] = W * lam["I11"]
    m[4::5] = W * lam["m11"]
    return m


def rect_nodes(ax: float, ay: float, order: int = 5) -> np.ndarray:
    n = order + 1
    x, _ = gll_points(n)
    X, Y = np.meshgrid((x + 1) / 2 * ax, (x + 1) / 2 * ay)
    return np.stack([X.reshape(-1), Y.reshape(-1)], axis=1)


def max_eigenvalue(xy: np.ndarray, lam: dict, order: int = 5) -> float:
    K = element_stiffness(xy, lam, order)
    m = element_mass(xy, lam, order)
    s = 1.0 / np.sqrt(m)
    ev = sla.eigvalsh(s[:, None] * K * s[None, :])
    return float(ev[-1])


def stable_dt(xy_list, lam_list, safety: float = 0.9, order: int = 5) -> float:
    """safety * 2/sqrt(max over elements of lambda_max(M_e^-1 K_e))."""
    lmax = max(max_eigenvalue(xy, lam, order) for xy in xy_list for lam in lam_list)
    return safety * 2.0 / np.sqrt(lmax)


def solid_element_matrices(xyz: np.ndarray, drow: np.ndarray, order: int = 5, nz: int = 3):
    """Dense stiffness (3*N square, DOF order u v w per node) and lumped mass
    of a 3D solid element with nodes xyz [N, 3] (x fastest, then y, then z),
    material row (D11 D12 D13 D14 D22 D23 D24 D33 D34 D44 D55 D56 D66 rho)."""
    n = order + 1
    _, w, D = gll_derivative_matrix(n)
    _, w3, D3 = gll_derivative_matrix(nz)
    I6, I3 = np.eye(n), np.eye(nz)
    ops = [np.kron(I3, np.kron(I6, D)), np.kron(I3, np.kron(D, I6)), np.kron(D3, np.kron(I6, I6))]
    W = np.kron(w3, np.kron(w, w))
    N = n * n * nz
    J = np.stack([np.stack([op @ xyz[:, b] for op in ops], -1) for b in range(3)], axis=1)  # [q, b, a]
    det = np.linalg.det(J)
    inv = np.linalg.inv(J)                                  # [q, a, b] = dxi_a / dx_b
    dN = np.stack(ops, axis=1)                              # [q, a, node]
    grad = np.einsum("qab,qan->qbn", inv, dN)               # [q, b, node]
    d = drow
    Dm = np.array([[d[0], d[1], d[2], d[3], 0, 0], [d[1], d[4], d[5], d[6], 0, 0], [d[2], d[5], d[7], d[8], 0, 0],
                   [d[3], d[6], d[8], d[9], 0, 0], [0, 0, 0, 0, d[10], d[11]], [0, 0, 0, 0, d[11], d[12]]])
    B = np.zeros((N, 6, 3 * N))
    gx, gy, gz = grad[:, 0], grad[:, 1], grad[:, 2]
    B[:, 0, 0::3], B[:, 1, 1::3], B[:, 2, 2::3] = gx, gy, gz
    B[:, 3, 0::3], B[:, 3, 1::3] = gy, gx          # xy
    B[:, 4, 1::3], B[:, 4, 2::3] = gz, gy          # yz
    B[:, 5, 0::3], B[:, 5, 2::3] = gz, gx          # xz
    DB = np.einsum("st,qtj->qsj", Dm, B, optimize=True)
    K = np.einsum("qsi,qsj->ij", B * (W * np.abs(det))[:, None, None], DB, optimize=True)
    m = np.repeat(W * np.abs(det) * d[13], 3)
    return K, m


def solid_stable_dt(xyz: np.ndarray, drows, safety: float = 0.9) -> float:
    lmax = 0.0
    for drow in drows:
        K, m = solid_element_matrices(xyz, np.asarray(drow, float))
        s = 1.0 / np.sqrt(m)
        lmax = max(lmax, float(sla.eigvalsh(s[:, None] * K * s[None, :])[-1]))
    return safety * 2.0 / np.sqrt(lmax)
