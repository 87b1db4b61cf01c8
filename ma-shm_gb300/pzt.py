"""PZT transducers: equivalent actuator loads and sensor constants (host, FP64).

The reference models a surface-bonded PZT disc as 3D piezoelectric spectral
elements (order 5 in plane, 3 GLL nodes through the PZT thickness) stacked on
the plate elements it covers (src/models/flat_shell/mesher/
connect_pzt3D_to_plate_fun.m, flat_shell_engine/coupl3D_global.m).  With the
bottom electrode at 0 V and the top at V0, the internal potential follows
from the static condensation of the dielectric matrix, and the piezoelectric
coupling turns it into nodal forces; the in-plane forces of the bottom layer
at the patch perimeter are applied to the plate as forces and moments about
the mid-plane with lever h/2 + t/2 (main_flat_shell.m:144-225).  This module
computes the same loads with its own element integration: tensor-product
Lagrange derivative matrices at the GLL points, element matrices for all
quadrature points at once, sparse assembly and a sparse solve.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sps
import scipy.sparse.linalg as spla

from .element import gll_derivative_matrix


def _lagrange_d(n):
    x, w, D = gll_derivative_matrix(n)
    return x, w, D


def piezo_element(xyz: np.ndarray, e_mat: np.ndarray, eps: np.ndarray, nxy: int = 6, nz: int = 3):
    """Coupling K_u,phi [3N x N] and dielectric K_phi,phi [N x N] of one 3D
    element.  xyz: [N, 3] node coordinates, node order x fastest, then y,
    then z (N = nxy*nxy*nz).  e_mat: 3x6 stress constants in strain order
    (xx, yy, zz, xy, yz, xz); eps: 3x3 permittivity."""
    _, w6, D6 = _lagrange_d(nxy)
    _, w3, D3 = _lagrange_d(nz)
    I6, I3 = np.eye(nxy), np.eye(nz)
    # derivative operators over the element nodes (row = quadrature node)
    Dxi = np.kron(I3, np.kron(I6, D6))
    Deta = np.kron(I3, np.kron(D6, I6))
    Dzeta = np.kron(D3, np.kron(I6, I6))
    W = np.kron(w3, np.kron(w6, w6))
    N = nxy * nxy * nz
    J = np.stack([np.stack([Dxi @ xyz[:, c] for c in range(3)], -1),
                  np.stack([Deta @ xyz[:, c] for c in range(3)], -1),
                  np.stack([Dzeta @ xyz[:, c] for c in range(3)], -1)], axis=1)   # [q, a, b] = dx_b/dxi_a
    det = np.linalg.det(J)
    inv = np.linalg.inv(J)                                                       # [q, b, a]
    dN = np.stack([Dxi, Deta, Dzeta], axis=1)                                    # [q, a, node]
    grad = np.einsum("qba,qan->qbn", inv, dN)                                    # [q, x/y/z, node]
    # local electric frame: v3 normal to the xi-eta tangents, v1 along xi
    t1, t2 = J[:, 0, :], J[:, 1, :]
    v3 = np.cross(t1, t2)
    v3 /= np.linalg.norm(v3, axis=1, keepdims=True)
    v1 = t1 / np.linalg.norm(t1, axis=1, keepdims=True)
    v2 = np.cross(v3, v1)
    v2 /= np.linalg.norm(v2, axis=1, keepdims=True)
    R = np.stack([v1, v2, v3], axis=1)                                           # [q, k, x]
    E = np.einsum("qkx,qxn->qkn", R, grad)                                       # field operator
    B = np.zeros((N, 6, 3 * N))
    gx, gy, gz = grad[:, 0, :], grad[:, 1, :], grad[:, 2, :]
    B[:, 0, 0::3] = gx
    B[:, 1, 1::3] = gy
    B[:, 2, 2::3] = gz
    B[:, 3, 0::3] = gy
    B[:, 3, 1::3] = gx
    B[:, 4, 1::3] = gz
    B[:, 4, 2::3] = gy
    B[:, 5, 0::3] = gz
    B[:, 5, 2::3] = gx
    wq = W * det
    Kup = np.einsum("q,qsi,ks,qkn->in", wq, B, e_mat, E)
    Kpp = np.einsum("q,qkm,kl,qln->mn", wq, E, eps, E)
    return Kup, Kpp


def patch_perimeter_nodes(nodes1: np.ndarray, elems: np.ndarray, n: int = 6) -> np.ndarray:
    """1-based plate nodes on the perimeter of an element patch: the nodes
    of element edges that belong to one element of the patch only."""
    edges = {}
    loc = [list(range(n)), [k * n + n - 1 for k in range(n)], list(range(n * n - n, n * n)),
           [k * n for k in range(n)]]
    for e in elems:
        for ed in loc:
            key = tuple(sorted(int(nodes1[e, c]) for c in ed))
            edges[key] = edges.get(key, 0) + 1
    per = set()
    for key, cnt in edges.items():
        if cnt == 1:
            per.update(key)
    return np.array(sorted(per), dtype=np.int64)


def actuator_loads(mesh: dict, elems, t_pzt: float, h: float, V0: float, e_mat: np.ndarray, eps: np.ndarray,
                   n: int = 6, nz: int = 3) -> np.ndarray:
    """Equivalent nodal load vector Fa [5*nnode] (reference DOF order) of a
    PZT patch covering the plate elements ``elems`` (0-based) driven at V0."""
    nodes1 = np.asarray(mesh["nodes"])
    coords = np.asarray(mesh["coords"], float)
    elems = np.asarray(elems, dtype=np.int64)
    zgll, _, _ = _lagrange_d(nz)
    patch = np.unique(nodes1[elems])               # plate nodes under the PZT (1-based)
    pidx = {int(g): i for i, g in enumerate(patch)}
    npn = len(patch)
    ntot = nz * npn                                # 3D nodes: layer-major
    rows_u, cols_u, vals_u, rows_p, cols_p, vals_p = [], [], [], [], [], []
    for e in elems:
        pl = np.array([pidx[int(g)] for g in nodes1[e]])
        gid = np.concatenate([pl + l * npn for l in range(nz)])
        xyz = np.zeros((n * n * nz, 3))
        for l in range(nz):
            sl = slice(l * n * n, (l + 1) * n * n)
            xyz[sl, 0] = coords[nodes1[e] - 1, 0]
            xyz[sl, 1] = coords[nodes1[e] - 1, 1]
            xyz[sl, 2] = coords[nodes1[e] - 1, 2] + h / 2 + (zgll[l] + 1) / 2 * t_pzt
        Kup, Kpp = piezo_element(xyz, e_mat, eps, n, nz)
        dof = (3 * gid[:, None] + np.arange(3)[None, :]).reshape(-1)
        rows_u.append(np.repeat(dof, len(gid)))
        cols_u.append(np.tile(gid, len(dof)))
        vals_u.append(Kup.reshape(-1))
        rows_p.append(np.repeat(gid, len(gid)))
        cols_p.append(np.tile(gid, len(gid)))
        vals_p.append(Kpp.reshape(-1))
    Kup = sps.csr_matrix((np.concatenate(vals_u), (np.concatenate(rows_u), np.concatenate(cols_u))),
                         shape=(3 * ntot, ntot))
    Kpp = sps.csr_matrix((np.concatenate(vals_p), (np.concatenate(rows_p), np.concatenate(cols_p))),
                         shape=(ntot, ntot))
    bottom = np.arange(npn)
    top = np.arange((nz - 1) * npn, nz * npn)
    inner = np.arange(npn, (nz - 1) * npn)
    phi = np.zeros(ntot)
    phi[top] = V0
    rhs = -(Kpp[inner][:, top] @ phi[top])
    phi[inner] = spla.spsolve(Kpp[inner][:, inner].tocsc(), rhs)
    F3 = Kup @ phi                                 # forces on the 3D nodes
    per = patch_perimeter_nodes(nodes1, elems, n)
    nnode = coords.shape[0]
    Fa = np.zeros(5 * nnode)
    for g in per:
        i = pidx[int(g)]                           # bottom-layer 3D node of plate node g
        fx, fy = F3[3 * bottom[i]], F3[3 * bottom[i] + 1]
        Fa[5 * (g - 1) + 0] = fx
        Fa[5 * (g - 1) + 2] = fy
        Fa[5 * (g - 1) + 1] = fx * (h / 2 + t_pzt / 2)
        Fa[5 * (g - 1) + 3] = fy * (h / 2 + t_pzt / 2)
    return Fa
