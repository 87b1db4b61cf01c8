"""Synthetic workloads with the shapes of the engine's reference configurations.

No measured or published dataset is involved; every plate, damage map and
excitation is generated here from a seed.  Sizes:

* ``plate_force``  (config "cfg1"): 0.5 m square CFRP plate, 20x20 order-5
  elements, 5-cycle Hann 50 kHz transverse force at the centre node, free
  edges, 0.5 ms, 8 out-of-plane outputs on a 150 mm circle.  FP64.
* ``plate_pzt``    (config "cfg2"): 1 m plate, 200x200 elements (~1 M nodes,
  ~5 M DOF), PZT disc 10 mm x 0.2 mm at the centre as electromechanical nodal
  loads, 100 kHz burst, 1 ms, w-velocity frames every 100 steps, 16 outputs.
* ``batch``        (config "cfg4"): 512 plates, side ~ U{40..80} elements of
  6.25 mm, 1-3 elliptical damage zones with stiffness reduction U(0.2, 0.8),
  random actuator node, carrier in {50, 75, 100} kHz, 8 outputs, 0.4 ms.  FP32.
* ``adjoint``      (config "cfg5"): 50x50 plate, 2 500 per-element damage
  parameters, hidden map with two zones at 0.5 reduction, 50 kHz.

Damping is the reference's usual mass-proportional pair (etad_xy = 4e2,
etad_z = 4e3 1/s, inputs/input16.m) and the time step is 0.9 x the element
eigenvalue bound (element.stable_dt).
"""
from __future__ import annotations

import numpy as np

from . import element as EL
from . import materials as M
from . import mesh as MS
from .solver import RunConfig, Scenario, hanning_signal

ETA_XY, ETA_Z = 4e2, 4e3


def _dt_for(ax, ay, lams):
    return EL.stable_dt([EL.rect_nodes(ax, ay)], lams)


def plate_force(nex=20, ney=20, L=0.5, T=0.5e-3, f=50e3, n_out=8, radius=0.15, dt=None, nft=None):
    lam = M.cfrp_laminate()
    mesh = MS.structured_plate(L, L, nex, ney)
    if dt is None:
        dt = _dt_for(L / nex, L / ney, [lam])
    if nft is None:
        nft = int(np.ceil(T / dt)) + 1
    xc = yc = L / 2
    centre = MS.nearest_node(mesh["coords"], xc, yc)
    outs = MS.circle_sensor_nodes(mesh, xc, yc, min(radius, 0.45 * L), n_out)
    _, st = hanning_signal(dt, nft, f / 5, f, 0.0)
    sc = Scenario(mesh=mesh, mat_table=M.table_row(lam)[None, :],
                  force_dof=np.array([5 * centre], np.int32), force_val=np.array([1.0]),
                  out_dof=(5 * outs).astype(np.int32), signal=st)
    run = RunConfig(dt=dt, nft=nft, nn_first=2, eta_xy=ETA_XY, eta_z=ETA_Z, h=lam["h"])
    return [sc], run


def plate_delamination(nex=20, ney=20, L=0.5, T=0.5e-3, f=50e3, zone=(0.32, 0.30, 0.06, 0.035, 0.5),
                       layer=4, n_out=8, radius=0.15, nft=None):
    """Plate of ``plate_force`` with one delamination between plies ``layer``
    and ``layer + 1`` (counted from the top surface) under an elliptical zone
    (xc, yc, a, b, angle in m / rad): the zone's elements are split into the
    sub-laminate above (plies 0..layer-1) and under (plies layer..) the
    delamination (split_delam_nodes_flat_shell.m, composite_plate_c_delam.m:88-173),
    both integrated about the intact laminate's mid-plane."""
    lam = M.cfrp_laminate()
    q = M.ply_stiffness(**M.CFRP_PLY)
    nply = len(M.CFRP_PLY_T)
    above = M.laminate(q, M.CFRP_RHO, M.CFRP_PLY_T, M.CFRP_ANGLES, plies=range(layer))
    under = M.laminate(q, M.CFRP_RHO, M.CFRP_PLY_T, M.CFRP_ANGLES, plies=range(layer, nply))
    base = MS.structured_plate(L, L, nex, ney)
    den = MS.elements_in_ellipse(base, *zone)
    nodes, coords, den_under, den_above = MS.split_delam_nodes_flat_shell(base["nodes"], base["coords"], den,
                                                                          MS.boundary_nodes(base))
    mesh = dict(nodes=nodes, coords=coords, structured=False, mesh_min=base["mesh_min"],
                mesh_max=base["mesh_max"], den_under=den_under, den_above=den_above, base=base)
    elem_mat = np.zeros(nodes.shape[0], np.int32)
    elem_mat[den_under] = 2
    elem_mat[den_above] = 1
    table = np.stack([M.table_row(lam), M.table_row(above), M.table_row(under)])
    dt = _dt_for(L / nex, L / ney, [lam, above, under])
    if nft is None:
        nft = int(np.ceil(T / dt)) + 1
    centre = MS.nearest_node(base["coords"], L / 2, L / 2)
    outs = MS.circle_sensor_nodes(base, L / 2, L / 2, min(radius, 0.45 * L), n_out)
    _, st = hanning_signal(dt, nft, f / 5, f, 0.0)
    sc = Scenario(mesh=mesh, mat_table=table, elem_mat=elem_mat,
                  force_dof=np.array([5 * centre], np.int32), force_val=np.array([1.0]),
                  out_dof=(5 * outs).astype(np.int32), signal=st)
    run = RunConfig(dt=dt, nft=nft, nn_first=2, eta_xy=ETA_XY, eta_z=ETA_Z, h=lam["h"])
    return [sc], run


def random_plate(rng, edge=6.25e-3, nmin=40, nmax=80, lam=None, n_out=8, freqs=(50e3, 75e3, 100e3),
                 dt=None, nft=None):
    """One scenario of the batched workload (damage zones, actuator, carrier)."""
    lam = lam or M.cfrp_laminate()
    nex = int(rng.integers(nmin, nmax + 1))
    ney = int(rng.integers(nmin, nmax + 1))
    mesh = MS.structured_plate(nex * edge, ney * edge, nex, ney)
    keep = np.ones(nex * ney)
    for _ in range(int(rng.integers(1, 4))):
        xc = rng.uniform(0.15, 0.85) * nex * edge
        yc = rng.uniform(0.15, 0.85) * ney * edge
        a = rng.uniform(5, 20) * edge / 2.5
        b = rng.uniform(5, 20) * edge / 2.5
        d = rng.uniform(0.2, 0.8)
        sel = MS.elements_in_ellipse(mesh, xc, yc, a, b, rng.uniform(0, np.pi))
        keep[sel] = 1.0 - d
    ax_ = MS.nearest_node(mesh["coords"], rng.uniform(0.2, 0.8) * nex * edge, rng.uniform(0.2, 0.8) * ney * edge)
    outs = MS.circle_sensor_nodes(mesh, nex * edge / 2, ney * edge / 2, 0.35 * min(nex, ney) * edge, n_out,
                                  phase=rng.uniform(0, np.pi))
    f = float(rng.choice(freqs))
    sc = Scenario(mesh=mesh, mat_table=M.table_row(lam)[None, :], elem_keep=keep,
                  force_dof=np.array([5 * ax_], np.int32), force_val=np.array([1.0]),
                  out_dof=(5 * outs).astype(np.int32))
    sc.carrier = f
    return sc


def batch(n=512, seed=0, T=0.4e-3, edge=6.25e-3, nmin=40, nmax=80, nft=None):
    lam = M.cfrp_laminate()
    rng = np.random.default_rng(seed)
    dt = _dt_for(edge, edge, [lam])
    if nft is None:
        nft = int(np.ceil(T / dt)) + 1
    scs = []
    for s in range(n):
        sc = random_plate(np.random.default_rng([seed, s]), edge, nmin, nmax, lam)
        _, sc.signal = hanning_signal(dt, nft, sc.carrier / 5, sc.carrier, 0.0)
        scs.append(sc)
    run = RunConfig(dt=dt, nft=nft, nn_first=2, eta_xy=ETA_XY, eta_z=ETA_Z, h=lam["h"])
    return scs, run


def dof_count(scenarios) -> int:
    return int(sum(5 * np.asarray(s.mesh["coords"]).shape[0] for s in scenarios))


def adjoint_maps(n=64, nex=50, L=0.5, nft=20000, f=50e3, seed=0, n_out=8):
    """Damage-identification batch: n plates with hidden maps of two
    elliptical zones at 50 % stiffness reduction; the model starts undamaged.
    Returns (model scenarios, run, hidden keep vectors)."""
    lam = M.cfrp_laminate()
    mesh = MS.structured_plate(L, L, nex, nex)
    dt = _dt_for(L / nex, L / nex, [lam])
    _, st = hanning_signal(dt, nft, f / 5, f, 0.0)
    fen = nex * nex
    centre = MS.nearest_node(mesh["coords"], L / 2, L / 2)
    outs = MS.circle_sensor_nodes(mesh, L / 2, L / 2, 0.3 * L, n_out)
    scs, hidden = [], []
    for s in range(n):
        rng = np.random.default_rng([seed, s])
        keep = np.ones(fen)
        for _ in range(2):
            xc, yc = rng.uniform(0.2, 0.8, 2) * L
            a, b = rng.uniform(0.03, 0.08, 2) * L
            keep[MS.elements_in_ellipse(mesh, xc, yc, a, b, rng.uniform(0, np.pi))] = 0.5
        hidden.append(keep)
        scs.append(Scenario(mesh=mesh, mat_table=M.table_row(lam)[None, :], elem_keep=np.ones(fen),
                            force_dof=np.array([5 * centre], np.int32), force_val=np.array([1.0]),
                            out_dof=(5 * outs).astype(np.int32), signal=st))
    run = RunConfig(dt=dt, nft=nft, nn_first=2, eta_xy=ETA_XY, eta_z=ETA_Z, h=lam["h"])
    return scs, run, hidden


def plate_pzt(nex=200, L=1.0, T=1e-3, f=100e3, d_pzt=10e-3, t_pzt=0.2e-3, V0=100.0, n_out=16, radius=0.15,
              frames_every=100, nft=None):
    """Config 2: plate with a centred PZT disc acting as actuator (equivalent
    electromechanical loads, pzt.actuator_loads) and as sensor (voltage),
    w-velocity frames every ``frames_every`` steps, ``n_out`` point outputs."""
    from . import pzt as PZ
    lam = M.cfrp_laminate()
    mesh = MS.structured_plate(L, L, nex, nex)
    p = M.pzt5a()
    pm = M.pzt_material(p["S"], p["d"], p["epsT"], 0.0)
    elems = MS.elements_in_disc(mesh, L / 2, L / 2, d_pzt / 2)
    lam_p = M.add_piezo_layer(lam, pm["Qpzt"], p["rho"], t_pzt)
    table = np.stack([M.table_row(lam), M.table_row(lam_p)])
    elem_mat = np.zeros(nex * nex, np.int32)
    elem_mat[elems] = 1
    Fa = PZ.actuator_loads(mesh, elems, t_pzt, lam["h"], V0, pm["epzt"], pm["gpzt"])
    nzi = np.nonzero(Fa)[0]
    dt = _dt_for(L / nex, L / nex, [lam, lam_p])
    if nft is None:
        nft = int(np.ceil(T / dt)) + 1
    _, st = hanning_signal(dt, nft, f / 5, f, 0.0)
    outs = MS.circle_sensor_nodes(mesh, L / 2, L / 2, min(radius, 0.45 * L), n_out)
    sc = Scenario(mesh=mesh, mat_table=table, elem_mat=elem_mat, force_dof=(nzi + 1).astype(np.int32),
                  force_val=Fa[nzi], out_dof=(5 * outs).astype(np.int32), signal=st, sensors=[elems],
                  pzt=dict(pzt_thickness=t_pzt, g33=pm["g33"], e31=pm["e31"], e32=pm["e32"]))
    run = RunConfig(dt=dt, nft=nft, nn_first=1, eta_xy=ETA_XY, eta_z=ETA_Z, h=lam["h"], frm_int=frames_every,
                    frame_dof=5)
    return [sc], run


def solid_plate(nex=120, L=0.5, T=0.5e-3, f=50e3, seed=0, n_out=8, radius=0.15, delam=True, nft=None,
                shear_as_reference=True):
    """Config 3: CFRP [0/90/45/-45]s plate as 3D solid elements, one element
    per ply (order 5 in plane, order 2 through the ply), per-ply rotated
    stiffness, a seeded elliptical delamination (semi-axes U(5, 20) mm) as
    split interface nodes between two plies, 50 kHz Hann burst as a
    transverse force at the top-surface centre, ``n_out`` w outputs on the
    top surface."""
    from .solver import SolidScenario
    rng = np.random.default_rng(seed)
    ply_t = np.array(M.CFRP_PLY_T)
    angles = np.array(M.CFRP_ANGLES)
    mesh = MS.solid_plate(L, L, nex, nex, ply_t)
    C = M.cfrp_c3d()
    # element layer i is the i-th ply from the bottom; plies are listed from the top
    rows = np.stack([M.solid_row(M.ply_c3d_rotated(C, angles[len(angles) - 1 - i]), M.CFRP_RHO, shear_as_reference)
                     for i in range(len(ply_t))])
    elem_mat = mesh["ply_layer_of_element"].astype(np.int32)
    info = {}
    if delam:
        a, b = rng.uniform(5e-3, 20e-3, 2)
        xc, yc = rng.uniform(0.25, 0.75, 2) * L
        interface = int(rng.integers(0, len(ply_t) - 1))
        els = MS.elements_in_ellipse(mesh["base"], xc, yc, a, b, rng.uniform(0, np.pi))
        if len(els):
            mesh = MS.split_interface(mesh, interface, els)
        info = dict(a=a, b=b, xc=xc, yc=yc, interface=interface, n_split=len(mesh.get("split_nodes", [])))
    xyz = np.zeros((108, 3))
    ax = L / nex
    g6, _ = MS.gll_points(6)
    g3, _ = MS.gll_points(3)
    for c in range(108):
        xyz[c] = ((g6[c % 6] + 1) / 2 * ax, (g6[(c // 6) % 6] + 1) / 2 * ax, (g3[c // 36] + 1) / 2 * ply_t[0])
    dt = EL.solid_stable_dt(xyz, rows)
    if nft is None:
        nft = int(np.ceil(T / dt)) + 1
    _, st = hanning_signal(dt, nft, f / 5, f, 0.0)
    NXY = mesh["NXY"]
    top = (mesh["nz"] - 1) * mesh["nply"] * NXY          # first node of the top node layer (0-based)
    base = mesh["base"]
    centre = MS.nearest_node(base["coords"], L / 2, L / 2) + top
    outs = MS.circle_sensor_nodes(base, L / 2, L / 2, min(radius, 0.45 * L), n_out) + top
    sc = SolidScenario(mesh=mesh, mat_table=rows, elem_mat=elem_mat,
                       force_dof=np.array([3 * centre], np.int32), force_val=np.array([1.0]),
                       out_dof=(3 * outs).astype(np.int32), signal=st)
    sc.delam = info
    run = RunConfig(dt=dt, nft=nft, nn_first=2, eta_xy=ETA_XY, eta_z=ETA_Z, h=float(ply_t.sum()))
    return [sc], run


def pressure_from_grid(data: np.ndarray, coords: np.ndarray, Lx: float = 0.5, Ly: float = 0.5) -> np.ndarray:
    """Nodal pressure frames [nframes, nnode] from gridded frames ``data``
    [ny, nx, nframes] spanning [0, Lx] x [0, Ly] (the Data array that
    main_flat_shell_pressure_excit_c.m:65-82 loads; its first index runs
    along y).  The reference interpolates with MATLAB's scatteredInterpolant
    (linear on a Delaunay triangulation of the grid, whose diagonal choice on a
    regular grid is arbitrary); this uses bilinear interpolation, which equals
    it wherever the field is linear inside a cell."""
    data = np.asarray(data, float)
    ny, nx, nf = data.shape
    fx = np.clip(coords[:, 0] / Lx * (nx - 1), 0, nx - 1)
    fy = np.clip(coords[:, 1] / Ly * (ny - 1), 0, ny - 1)
    i0 = np.minimum(fx.astype(int), nx - 2)
    j0 = np.minimum(fy.astype(int), ny - 2)
    ax, ay = fx - i0, fy - j0
    out = np.empty((nf, coords.shape[0]))
    for k in range(nf):
        d = data[:, :, k]
        out[k] = ((1 - ax) * (1 - ay) * d[j0, i0] + ax * (1 - ay) * d[j0, i0 + 1] +
                  (1 - ax) * ay * d[j0 + 1, i0] + ax * ay * d[j0 + 1, i0 + 1])
    return out


def plate_pressure(nex=10, ney=10, L=0.1, nft=400, f=200e3, npf=25, p0=1e3, seed=0):
    """Plate loaded by a moving Gaussian pressure spot (a synthetic stand-in for
    the COMSOL pressure field of main_flat_shell_pressure_excit_c.m), frames on
    a 41x41 grid every few time steps, dt and the loop as the _c variants
    (dt = tt/(nft-1), nn = 1..nft)."""
    lam = M.cfrp_laminate()
    mesh = MS.structured_plate(L, L, nex, ney)
    dt = _dt_for(L / nex, L / ney, [lam])
    tt = dt * (nft - 1)
    g = np.linspace(0.0, L, 41)
    X, Y = np.meshgrid(g, g)
    times = np.linspace(0.0, 0.8 * tt, npf)
    rng = np.random.default_rng(seed)
    x0, y0 = rng.uniform(0.3, 0.7, 2) * L
    data = np.empty((41, 41, npf))
    for k, t in enumerate(times):
        w = np.sin(2 * np.pi * f * t) * np.exp(-((X - x0 - 0.2 * L * t / tt) ** 2 + (Y - y0) ** 2) / (0.05 * L) ** 2)
        data[:, :, k] = p0 * w
    nodal = pressure_from_grid(data, mesh["coords"], L, L)
    outs = MS.circle_sensor_nodes(mesh, L / 2, L / 2, 0.3 * L, 6)
    sc = Scenario(mesh=mesh, mat_table=M.table_row(lam)[None, :], out_dof=(5 * outs).astype(np.int32),
                  signal=np.zeros(nft), pressure=dict(times=times, nodal=nodal))
    run = RunConfig(dt=dt, nft=nft, nn_first=1, eta_xy=ETA_XY, eta_z=ETA_Z, h=lam["h"])
    return [sc], run


def plate_multi_pzt(nex=40, L=0.2, n_pzt=3, actuator_no=2, d_pzt=10e-3, t_pzt=0.2e-3, V0=100.0, nft=600,
                    f=150e3, random=False, seed=0):
    """main_flat_shell_multi_pzt_c.m: n_pzt PZT discs on a circle, all bonded
    (PZT layer in their elements) and all sensors; disc ``actuator_no``
    (1-based) is driven (:150-230).  ``random`` drives it with white noise
    (main_flat_shell_multi_pzt_c_random_exc_signals.m:137-139) instead of the
    Hann burst."""
    from . import pzt as PZ
    from .solver import random_signal
    lam = M.cfrp_laminate()
    mesh = MS.structured_plate(L, L, nex, nex)
    p = M.pzt5a()
    pm = M.pzt_material(p["S"], p["d"], p["epsT"], 0.0)
    lam_p = M.add_piezo_layer(lam, pm["Qpzt"], p["rho"], t_pzt)
    ang = 2 * np.pi * np.arange(n_pzt) / n_pzt
    discs = [MS.elements_in_disc(mesh, L / 2 + 0.25 * L * np.cos(a), L / 2 + 0.25 * L * np.sin(a), d_pzt / 2)
             for a in ang]
    elem_mat = np.zeros(nex * nex, np.int32)
    for d in discs:
        elem_mat[d] = 1
    Fa = PZ.actuator_loads(mesh, discs[actuator_no - 1], t_pzt, lam["h"], V0, pm["epzt"], pm["gpzt"])
    nzi = np.nonzero(Fa)[0]
    dt = _dt_for(L / nex, L / nex, [lam, lam_p])
    st = random_signal(nft, seed) if random else hanning_signal(dt, nft, f / 5, f, 0.0)[1]
    centre = MS.nearest_node(mesh["coords"], L / 2, L / 2)
    sc = Scenario(mesh=mesh, mat_table=np.stack([M.table_row(lam), M.table_row(lam_p)]), elem_mat=elem_mat,
                  force_dof=(nzi + 1).astype(np.int32), force_val=Fa[nzi],
                  out_dof=np.array([5 * centre], np.int32), signal=st, sensors=discs,
                  pzt=dict(pzt_thickness=t_pzt, g33=pm["g33"], e31=pm["e31"], e32=pm["e32"]))
    run = RunConfig(dt=dt, nft=nft, nn_first=1, eta_xy=ETA_XY, eta_z=ETA_Z, h=lam["h"])
    return [sc], run
