"""Unstructured quad meshes to spectral elements, numbered as the reference does.

The reference meshes plates with gmsh, loads gmsh's MATLAB export
(``msh.POS``, ``msh.QUADS``, ...; automesh_delam.m:229), turns clockwise
quads around (change_turn_quad.m) and converts the 4-node quads into
order-N spectral elements (quad2spectral_Fiborek.m).  The engine takes the
resulting ``nodes``/``coords`` as they are, so the node numbering here follows
quad2spectral_Fiborek.m: corner nodes keep the quad numbering, edge-interior
nodes follow in the lexicographic order of their coordinates (MATLAB
``unique(...,'rows')``), then each element's interior nodes.
"""
from __future__ import annotations

import re

import numpy as np

from .mesh import gll_points


def read_gmsh_m(path: str) -> dict:
    """Arrays of a gmsh MATLAB export (``msh.NAME = [ rows ];`` blocks and
    scalar assignments such as ``msh.nbNod = 4;``)."""
    text = open(path).read()
    out = {}
    for m in re.finditer(r"msh\.(\w+)\s*=\s*\[(.*?)\];", text, flags=re.S):
        rows = [r for r in re.split(r"[;\n]", m.group(2)) if r.strip()]
        out[m.group(1)] = np.array([[float(v) for v in r.replace(",", " ").split()] for r in rows])
    for m in re.finditer(r"msh\.(\w+)\s*=\s*([-+0-9.eE]+)\s*;", text):
        out.setdefault(m.group(1), float(m.group(2)))
    return out


def change_turn_quad(quads: np.ndarray, pos: np.ndarray) -> np.ndarray:
    """Quads whose bilinear Jacobian determinant is not positive at some corner
    are renumbered 1,4,3,2 (change_turn_quad.m); 1-based node ids in and out."""
    q = np.asarray(quads, dtype=np.int64).copy()
    x = pos[q - 1, 0]
    y = pos[q - 1, 1]
    # corners 1..4 counter-clockwise; at corner c the edges to the next and the
    # previous corner span the Jacobian (up to positive factors)
    nxt, prv = [1, 2, 3, 0], [3, 0, 1, 2]
    det = np.stack([(x[:, nxt[c]] - x[:, c]) * (y[:, prv[c]] - y[:, c]) -
                    (y[:, nxt[c]] - y[:, c]) * (x[:, prv[c]] - x[:, c]) for c in range(4)], axis=1)
    bad = (det <= 0).any(axis=1)
    q[bad] = q[bad][:, [0, 3, 2, 1]]
    return q


def _round6(v: np.ndarray) -> np.ndarray:
    # MATLAB round (halves away from zero) to 1e-6, then * 1e-6
    return np.sign(v) * np.floor(np.abs(v) * 1e6 + 0.5) * 1e-6


def quad2spectral(quads: np.ndarray, pos: np.ndarray, order: int = 5):
    """4-node quads (1-based, counter-clockwise) and node coordinates [n, 3]
    to order-``order`` spectral elements: (nodes [fen, (order+1)^2] 1-based,
    local order xi fastest; coords [N, 3]; boundary_nodes 1-based)."""
    quads = np.asarray(quads, dtype=np.int64)
    pos = np.asarray(pos, dtype=float)
    if pos.shape[1] == 2:
        pos = np.concatenate([pos, np.zeros((pos.shape[0], 1))], axis=1)
    n = order + 1
    ni = n - 2
    fen = quads.shape[0]
    ksi, _ = gll_points(n)
    kin = ksi[1:n - 1]
    # element edges 1->2, 2->3, 3->4, 4->1: rounded midpoints and half lengths
    a = pos[quads - 1]                       # [fen, 4, 3]
    b = pos[quads[:, [1, 2, 3, 0]] - 1]
    mid = _round6((b + a) / 2)
    half = (b - a) / 2
    pts = mid[:, :, None, :] + half[:, :, None, :] * kin[None, None, :, None]   # [fen, 4, ni, 3]
    flat = pts.reshape(-1, 3)
    uniq, inv = np.unique(flat, axis=0, return_inverse=True)
    inv = inv.reshape(fen, 4, ni)
    ncorner = int(quads.max())
    nedge = uniq.shape[0]
    edge_id = inv + 1 + ncorner              # 1-based global ids
    # interior nodes: intersections of the lines edge1_k -> edge3_k and
    # edge4_m -> edge2_m (edges 3 and 4 read backwards)
    p1 = pts[:, 0]                           # [fen, ni, 3]
    p2 = pts[:, 1]
    p3 = pts[:, 2, ::-1]
    p4 = pts[:, 3, ::-1]
    A13 = p3[..., 1] - p1[..., 1]
    B13 = p1[..., 0] - p3[..., 0]
    C13 = (p1[..., 1] - p3[..., 1]) * p1[..., 0] + (p3[..., 0] - p1[..., 0]) * p1[..., 1]
    A42 = p2[..., 1] - p4[..., 1]
    B42 = p4[..., 0] - p2[..., 0]
    C42 = (p4[..., 1] - p2[..., 1]) * p4[..., 0] + (p2[..., 0] - p4[..., 0]) * p4[..., 1]
    # [fen, m (edge 4/2 index), k (edge 1/3 index)]
    W = A13[:, None, :] * B42[:, :, None] - B13[:, None, :] * A42[:, :, None]
    X = (B13[:, None, :] * C42[:, :, None] - C13[:, None, :] * B42[:, :, None]) / W
    Y = (C13[:, None, :] * A42[:, :, None] - A13[:, None, :] * C42[:, :, None]) / W
    zs = np.unique(uniq[:, 2])
    if zs.size != 1:
        raise ValueError("quad2spectral: the mesh must be planar (one z value)")
    interior = np.stack([X.reshape(-1), Y.reshape(-1), np.full(X.size, zs[0])], axis=1)
    int_id = (1 + ncorner + nedge + np.arange(fen * ni * ni)).reshape(fen, ni, ni)   # [e, m, k]
    nodes = np.zeros((fen, n, n), dtype=np.int64)                                  # [e, row, col]
    nodes[:, 0, 0], nodes[:, 0, n - 1] = quads[:, 0], quads[:, 1]
    nodes[:, n - 1, n - 1], nodes[:, n - 1, 0] = quads[:, 2], quads[:, 3]
    nodes[:, 0, 1:n - 1] = edge_id[:, 0]
    nodes[:, 1:n - 1, n - 1] = edge_id[:, 1]
    nodes[:, n - 1, 1:n - 1] = edge_id[:, 2, ::-1]
    nodes[:, 1:n - 1, 0] = edge_id[:, 3, ::-1]
    nodes[:, 1:n - 1, 1:n - 1] = int_id
    coords = np.concatenate([pos[:ncorner], uniq, interior])
    # boundary: edges whose rounded midpoint appears once
    _, mid_inv, cnt = np.unique(mid.reshape(-1, 3), axis=0, return_inverse=True, return_counts=True)
    on_bnd = (cnt[mid_inv] == 1).reshape(fen, 4)
    sides = [nodes[:, 0, :], nodes[:, :, n - 1], nodes[:, n - 1, :], nodes[:, :, 0]]
    bnd = np.unique(np.concatenate([sides[s][on_bnd[:, s]].reshape(-1) for s in range(4)]))
    return nodes.reshape(fen, n * n).astype(np.int32), coords, bnd.astype(np.int32)
