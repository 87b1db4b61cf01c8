"""Pressure loading (main_flat_shell_pressure_excit_c.m) on CPU: the oracle's
pressure term against point forces of the same size, and the grid-to-node
interpolation of the pressure frames.  GPU parity of the pressure-loaded
step is in test_flat_shell_gpu.py."""
import numpy as np

from oracle.oracle import OracleProblem


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def test_uniform_pressure_equals_lumped_point_forces(pkg):
    """A pressure p0 constant in space over [0, T] is the w load p0 * (sum of
    w_i w_j detJ over the node's element copies) switched on for t <= T."""
    scs, run = pkg.workloads.plate_pressure(nex=5, ney=4, L=0.05, nft=160)
    sc = scs[0]
    nn = sc.mesh["coords"].shape[0]
    T = 60 * run.dt
    p0 = 750.0
    orc = OracleProblem(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table)
    kw = dict(nn_first=1, eta_xy=run.eta_xy, eta_z=run.eta_z, out_dof=sc.out_dof, h=run.h)
    a = orc.run(run.dt, run.nft, np.zeros(run.nft), pressure=dict(times=[0.0, T], nodal=np.full((2, nn), p0)),
                **kw)
    area = np.zeros(nn)
    np.add.at(area, sc.mesh["nodes"].reshape(-1) - 1, orc.WWDetJ)
    st = ((np.arange(1, run.nft + 1) - 1) * run.dt <= T).astype(float)
    b = orc.run(run.dt, run.nft, st, force_dof=5 * np.arange(1, nn + 1), force_val=p0 * area, **kw)
    assert np.abs(a["displ"]).max() > 0
    # same load, summed in a different order (per local copy vs per node)
    assert rel(a["displ"], b["displ"]) <= 1e-10
    assert rel(a["U"], b["U"]) <= 1e-10


def test_pressure_outside_the_frames_is_zero(pkg):
    scs, run = pkg.workloads.plate_pressure(nex=4, ney=4, L=0.04, nft=80)
    sc = scs[0]
    nn = sc.mesh["coords"].shape[0]
    orc = OracleProblem(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table)
    late = dict(times=[1.0, 2.0], nodal=np.ones((2, nn)))   # frames long after the run
    r = orc.run(run.dt, run.nft, np.zeros(run.nft), nn_first=1, out_dof=sc.out_dof, pressure=late)
    assert np.abs(r["U"]).max() == 0.0


def test_grid_to_node_interpolation_is_exact_for_bilinear_fields(pkg):
    mesh = pkg.mesh.structured_plate(0.5, 0.5, 7, 5)
    g = np.linspace(0.0, 0.5, 21)
    X, Y = np.meshgrid(g, g)                      # Data(iy, ix): first index along y
    f = lambda x, y: 3.0 + 2.0 * x - 5.0 * y + 7.0 * x * y
    data = np.stack([f(X, Y), 2 * f(X, Y)], axis=2)
    nodal = pkg.workloads.pressure_from_grid(data, mesh["coords"])
    c = mesh["coords"]
    assert np.abs(nodal[0] - f(c[:, 0], c[:, 1])).max() <= 1e-12
    assert np.abs(nodal[1] - 2 * f(c[:, 0], c[:, 1])).max() <= 1e-12
