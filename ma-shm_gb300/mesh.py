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


def solid_plate(Lx: float, Ly: float, nex: int, ney: int, ply_t, order: int = 5, nz: int = 3) -> dict:
    """Laminate plate of 3D spectral elements, one element per ply through the
    thickness (order ``order`` in plane, ``nz`` GLL nodes through the ply),
    as extrude_mesh.m builds it: elements layer by layer (bottom ply first),
    local nodes x fastest then y then z, global nodes numbered node layer by
    node layer (in-plane row-major inside a layer).  z runs from -h/2 to +h/2."""
    base = structured_plate(Lx, Ly, nex, ney, order)
    ply_t = np.asarray(ply_t, float)
    nply = len(ply_t)
    zg, _ = gll_points(nz)
    NXY = base["coords"].shape[0]
    h = float(ply_t.sum())
    zb = -h / 2 + np.concatenate(([0.0], np.cumsum(ply_t)))
    nlay = (nz - 1) * nply + 1
    zl = np.empty(nlay)
    for i in range(nply):
        for k in range(nz):
            zl[(nz - 1) * i + k] = zb[i] + (zg[k] + 1) / 2 * ply_t[i]
    coords = np.zeros((nlay * NXY, 3))
    coords[:, 0] = np.tile(base["coords"][:, 0], nlay)
    coords[:, 1] = np.tile(base["coords"][:, 1], nlay)
    coords[:, 2] = np.repeat(zl, NXY)
    fen2 = base["nodes"].shape[0]
    nodes = np.zeros((nply * fen2, base["nodes"].shape[1] * nz), np.int32)
    npl = base["nodes"].shape[1]
    for i in range(nply):
        for k in range(nz):
            nodes[i * fen2:(i + 1) * fen2, k * npl:(k + 1) * npl] = base["nodes"] + ((nz - 1) * i + k) * NXY
    return dict(nodes=nodes, coords=coords, nex=nex, ney=ney, nply=nply, nz=nz, NXY=NXY, fen2=fen2,
                ply_layer_of_element=np.repeat(np.arange(nply), fen2), h=h, base=base)


def split_interface(mesh3d: dict, interface: int, elems2d) -> dict:
    """Delamination between ply layers ``interface`` and ``interface+1``
    (0-based from the bottom) under the in-plane elements ``elems2d``:
    interface nodes whose every adjacent in-plane element is delaminated get
    a copy, and the elements of the upper ply use the copies, so that the two
    plies are not connected there (the perimeter nodes stay shared).  This is
    the topology change of split_delam_nodes2.m; no stiffness is added."""
    nodes = mesh3d["nodes"].copy()
    coords = mesh3d["coords"]
    base = mesh3d["base"]
    nz, fen2, NXY = mesh3d["nz"], mesh3d["fen2"], mesh3d["NXY"]
    npl = base["nodes"].shape[1]
    delam = np.zeros(fen2, bool)
    delam[np.asarray(elems2d, int)] = True
    # in-plane nodes touched only by delaminated elements
    touched_bad = np.zeros(NXY + 1, bool)
    touched_good = np.zeros(NXY + 1, bool)
    for e in range(fen2):
        (touched_bad if delam[e] else touched_good)[base["nodes"][e]] = True
    inner = np.nonzero(touched_bad & ~touched_good)[0]          # 1-based in-plane node ids
    layer = (nz - 1) * (interface + 1)
    old = inner + layer * NXY                                   # 1-based global ids
    new = coords.shape[0] + 1 + np.arange(len(inner))
    remap = dict(zip(old.tolist(), new.tolist()))
    upper = slice((interface + 1) * fen2, (interface + 2) * fen2)
    blk = nodes[upper, :npl]                                    # bottom node layer of the upper ply
    flat = blk.reshape(-1)
    for i, g in enumerate(flat):
        r = remap.get(int(g))
        if r is not None:
            flat[i] = r
    nodes[upper, :npl] = flat.reshape(blk.shape)
    out = dict(mesh3d)
    out["nodes"] = nodes
    out["coords"] = np.concatenate([coords, coords[old - 1]])
    out["split_nodes"] = old
    return out


def boundary_nodes(mesh: dict) -> np.ndarray:
    """1-based ids of every node on the outer boundary of a structured plate,
    GLL edge nodes included (the ``boundary_nodes`` output of
    quad2spectral_Fiborek.m:156)."""
    NX, NY = mesh["NX"], mesh["NY"]
    g = np.arange(NX * NY).reshape(NY, NX)
    return np.unique(np.concatenate([g[0], g[-1], g[:, 0], g[:, -1]])) + 1


def split_delam_nodes_flat_shell(nodes: np.ndarray, coords: np.ndarray, den, boundary, order: int = 5):
    """Delamination topology of the flat shell (split_delam_nodes_flat_shell.m:37-268).

    The delaminated elements ``den`` (0-based) are duplicated: the originals
    become the sub-laminate under the delamination (``den_under``) and the
    copies, appended as elements fen, fen+1, ..., the one above it
    (``den_above``).  Nodes of the delaminated region are split (the copies
    get new ids with the same coordinates) except the region's outer nodes,
    which both sub-laminates and the intact plate keep sharing:

    * a corner node is outer when at most two delaminated elements have it as
      a corner (a corner shared by three, the inside of an L, counts as inner,
      as in the reference);
    * an edge node is outer when no other delaminated element has it on an edge;
    * outer nodes on the plate's boundary are split anyway, except the
      "free" corners (corner of a single delaminated element) lying on the
      boundary; with three of those the smallest id is split too.

    Counts are the reference's pairwise neighbour loops rewritten as
    occurrence counts (an element's own corner/edge positions hold a node at
    most once).  Inner nodes get new ids in ascending order of the old ids.
    Returns (nodes, coords, den_under, den_above) with 1-based node ids.
    """
    nodes = np.asarray(nodes)
    coords = np.asarray(coords, dtype=float)
    den = np.asarray(den, dtype=np.int64).reshape(-1)
    fen, npe = nodes.shape
    n = order + 1
    if npe != n * n:
        raise ValueError("nodes must have (order+1)^2 columns")
    loc = np.arange(npe).reshape(n, n)                              # [eta, xi]
    corner_pos = np.array([loc[0, 0], loc[0, -1], loc[-1, 0], loc[-1, -1]])
    edge_pos = np.concatenate([loc[0, 1:-1], loc[1:-1, -1], loc[-1, 1:-1], loc[1:-1, 0]])
    nm = int(nodes.max())
    sub = nodes[den]                                                # [nd, npe]
    cn = sub[:, corner_pos].reshape(-1)
    en = sub[:, edge_pos].reshape(-1)
    ccount = np.bincount(cn, minlength=nm + 1)
    ecount = np.bincount(en, minlength=nm + 1)
    outer = np.concatenate([cn[ccount[cn] <= 2], en[ecount[en] == 1]])
    free_corner = cn[ccount[cn] == 1]
    special = np.intersect1d(free_corner, np.asarray(boundary))
    if special.size == 3:
        special = special[1:]
    outer = np.union1d(np.setdiff1d(np.unique(outer), np.asarray(boundary)), special)
    inner = np.setdiff1d(np.unique(sub), outer)
    new_id = np.zeros(nm + 1, dtype=np.int64)
    new_id[inner] = nm + 1 + np.arange(inner.size)
    above = sub.copy()
    hit = new_id[above] > 0
    above[hit] = new_id[above[hit]]
    out_nodes = np.concatenate([nodes, above.astype(nodes.dtype)])
    nmax = nm + inner.size
    out_coords = np.zeros((nmax, coords.shape[1]))
    out_coords[:min(nm, coords.shape[0])] = coords[:nm]
    out_coords[above - 1] = out_coords[sub - 1]
    den_above = fen + np.arange(den.size)
    return out_nodes, out_coords, den.copy(), den_above
