"""Structured plate meshes in the reference's mesh format.

The reference meshes plates with gmsh and converts the quads to order-N
spectral elements (src/models/flat_shell/mesher/quad2spectral_Fiborek.m); the
solver then loads ``nodes`` [fen x (N+1)^2] (1-based) and ``coords``
[nnode x 3].  gmsh is outside this engine; ``structured_plate`` produces the
same arrays for rectangular plates meshed as nex x ney equal rectangles, with
the element-local node order the solver relies on (shape2D_prim.m:45-47:
local node c = k2*(N+1) + k1, xi fastest, xi along +x, eta along +y).
Global nodes are numbered row by row (x fastest), which is what the engine's
structured fused kernel recognises.
"""
from __future__ import annotations

import numpy as np


def gll_points(n: int):
    """GLL nodes/weights on [-1, 1]: endpoints + roots of P'_{n-1}."""
    if n < 2:
        raise ValueError("need at least 2 GLL points")
    N = n - 1
    # eigenvalues of the symmetric Jacobi matrix of the (1,1) Jacobi
    # polynomials give the interior points (Golub-Welsch)
    if N >= 2:
        k = np.arange(1, N - 1)
        b = np.sqrt(k * (k + 2.0) / ((2 * k + 1.0) * (2 * k + 3.0)))
        J = np.diag(b, 1) + np.diag(b, -1)
        inner = np.sort(np.linalg.eigvalsh(J))
    else:
        inner = np.zeros(0)
    x = np.concatenate(([-1.0], inner, [1.0]))
    x = 0.5 * (x - x[::-1])
    # Legendre P_N at the nodes by recurrence
    p0 = np.ones_like(x)
    p1 = x.copy()
    for m in range(2, N + 1):
        p0, p1 = p1, ((2 * m - 1) * x * p1 - (m - 1) * p0) / m
    w = 2.0 / (N * (N + 1) * p1 ** 2)
    return x, w


def structured_plate(Lx: float, Ly: float, nex: int, ney: int, order: int = 5, x0: float = 0.0,
                     y0: float = 0.0) -> dict:
    """Rectangular plate [x0, x0+Lx] x [y0, y0+Ly], nex x ney elements of order ``order``."""
    n = order + 1
    ksi, _ = gll_points(n)
    NX, NY = order * nex + 1, order * ney + 1
    ax, ay = Lx / nex, Ly / ney
    xs = np.empty(NX)
    ys = np.empty(NY)
    for ex in range(nex):
        xs[order * ex: order * ex + n] = x0 + ex * ax + (ksi + 1) / 2 * ax
    for ey in range(ney):
        ys[order * ey: order * ey + n] = y0 + ey * ay + (ksi + 1) / 2 * ay
    xs[-1] = x0 + Lx
    ys[-1] = y0 + Ly
    coords = np.zeros((NX * NY, 3))
    coords[:, 0] = np.tile(xs, NY)
    coords[:, 1] = np.repeat(ys, NX)
    ex = np.arange(nex)
    ey = np.arange(ney)
    k1 = np.arange(n)
    # nodes[e, c], e = ey*nex + ex, c = k2*n + k1
    base = (order * ey)[:, None] * NX + (order * ex)[None, :]            # [ney, nex]
    off = (k1[:, None] * NX + k1[None, :])                                 # [k2, k1]
    nodes = (base.reshape(-1, 1) + off.reshape(1, -1) + 1).astype(np.int32)
    return dict(nodes=nodes, coords=coords, nex=nex, ney=ney, NX=NX, NY=NY, ax=ax, ay=ay, order=order,
                Lx=Lx, Ly=Ly, x0=x0, y0=y0,
                mesh_min=np.array([x0, y0]), mesh_max=np.array([x0 + Lx, y0 + Ly]))


def nearest_node(coords: np.ndarray, x: float, y: float) -> int:
    """1-based node nearest to (x, y): ``[~,I]=min(sqrt(...))`` (main_flat_shell.m:45)."""
    d = np.sqrt((coords[:, 0] - x) ** 2 + (coords[:, 1] - y) ** 2)
    return int(np.argmin(d)) + 1


def element_centres(mesh: dict) -> np.ndarray:
    c = mesh["coords"][mesh["nodes"] - 1]
    return c[:, :, :2].mean(axis=1)


def elements_in_disc(mesh: dict, xc: float, yc: float, r: float) -> np.ndarray:
    """0-based elements whose centre lies inside the disc (PZT footprint)."""
    cen = element_centres(mesh)
    d = np.hypot(cen[:, 0] - xc, cen[:, 1] - yc)
    sel = np.nonzero(d <= r)[0]
    if sel.size == 0:
        sel = np.array([int(np.argmin(d))])
    return sel.astype(np.int32)


def elements_in_ellipse(mesh: dict, xc, yc, a, b, angle=0.0) -> np.ndarray:
    """0-based elements whose centre lies inside an ellipse (damage zones)."""
    cen = element_centres(mesh)
    ca, sa = np.cos(angle), np.sin(angle)
    dx, dy = cen[:, 0] - xc, cen[:, 1] - yc
    u = (ca * dx + sa * dy) / a
    v = (-sa * dx + ca * dy) / b
    return np.nonzero(u * u + v * v <= 1.0)[0].astype(np.int32)


def circle_sensor_nodes(mesh: dict, xc: float, yc: float, r: float, n: int, phase: float = 0.0):
    """1-based nodes nearest to n points evenly spaced on a circle."""
    ang = phase + 2 * np.pi * np.arange(n) / n
    return np.array([nearest_node(mesh["coords"], xc + r * np.cos(t), yc + r * np.sin(t)) for t in ang],
                    dtype=np.int32)
