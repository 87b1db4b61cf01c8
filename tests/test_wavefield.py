"""Wavefield-to-grid interpolation (spec2meshgrid_flat_shell.m) against the oracle.

CPU: the library's host set-up (grid points, owner elements, local
coordinates after three Newton steps) equals the oracle's restatement of the
reference: points and owners exactly, (ksi, eta) to 1e-11 (the oracle uses
the reference's inverse 2D Vandermonde matrix, the library the equivalent
tensor-product Lagrange basis).
GPU: the interpolation kernel against the oracle's Data for every motion
type and both surfaces (FP64, relative L2 <= 1e-10), from host frames and
from a plan's device-resident frames, plus exact reproduction of a degree-5
polynomial field on an affine mesh.
"""
import numpy as np
import pytest

from oracle import ref_setup as R

H = 3.9e-3


def _meshes(pkg):
    from tests.test_oracle_physics import _distorted
    out = {"structured": pkg.mesh.structured_plate(0.12, 0.1, 12, 10),
           "distorted": _distorted(pkg, nex=5, ney=4)}
    scs, _ = pkg.workloads.plate_delamination(nex=10, ney=10, L=0.1, T=1e-6, zone=(0.05, 0.05, 0.025, 0.015, 0.3),
                                              layer=3)
    out["delaminated"] = scs[0].mesh
    return out


def _oracle(mesh, n, fields, motion, surface):
    return R.spec2meshgrid_flat_shell(mesh["nodes"], mesh["coords"], n, n, fields, motion, surface, H,
                                      mesh.get("den_under", ()), mesh.get("den_above", ()))


@pytest.mark.parametrize("name", ["structured", "distorted", "delaminated"])
@pytest.mark.parametrize("n", [7, 33])
def test_grid_setup_matches_oracle(pkg, name, n):
    mesh = _meshes(pkg)[name]
    nn = mesh["coords"].shape[0]
    g = pkg.wavefield.Grid(mesh, n, n, "top", device=None)
    P = g.points()
    g.close()
    _, S = _oracle(mesh, n, {"x": np.zeros((1, nn))}, 1, "top")
    assert np.array_equal(P["xp"], S["xp"]) and np.array_equal(P["yp"], S["yp"])
    assert np.array_equal(P["owner"], S["owner"])
    assert np.abs(P["ksi"] - S["ksi_p"]).max() <= 1e-11
    assert np.abs(P["eta"] - S["eta_p"]).max() <= 1e-11
    assert P["max_err"] <= 1e-9


def test_grid_rejects_bad_arguments(pkg):
    mesh = _meshes(pkg)["structured"]
    with pytest.raises(pkg.native.ShmError):
        pkg.wavefield.Grid(mesh, 1, 5, device=None)
    with pytest.raises(ValueError):
        pkg.wavefield.Grid(mesh, 5, 5, surface="middle", device=None)
    g = pkg.wavefield.Grid(mesh, 5, 5, device=None)
    nn = mesh["coords"].shape[0]
    with pytest.raises(pkg.native.ShmError):   # host-only grid: no interpolation
        g.interpolate(np.zeros((1, 5, nn)), [0, 1, 2, 3, 4], 1, H)
    g.close()


def test_variable_names(pkg):
    vn = pkg.wavefield.variable_name
    assert vn("velocity", 3) == "Vz" and vn("displacement", 6) == "Ux_top"
    assert vn("acceleration", 8) == "accelerations_in_plane" and vn("velocity", 9) == "total_velocities"


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["structured", "distorted", "delaminated"])
def test_interpolation_matches_oracle_all_motions(pkg, name):
    mesh = _meshes(pkg)[name]
    nn = mesh["coords"].shape[0]
    rng = np.random.default_rng(3)
    frames = rng.standard_normal((3, 5, nn))
    comps = ("x", "Fix", "y", "Fiy", "z")
    fields = {c: frames[:, k] for k, c in enumerate(comps)}
    n = 24
    for surface in ("top", "bottom"):
        g = pkg.wavefield.Grid(mesh, n, n, surface)
        for motion in range(1, 10):
            got = g.interpolate(frames, [0, 1, 2, 3, 4], motion, H)       # [nframes, ny, nx]
            ref, _ = _oracle(mesh, n, fields, motion, surface)            # [ny, nx, nframes]
            assert rel(got, np.transpose(ref, (2, 0, 1))) <= 1e-10, (surface, motion)
        g.close()


@pytest.mark.gpu
def test_polynomial_field_reproduced(pkg):
    mesh = pkg.mesh.structured_plate(0.12, 0.1, 6, 5)
    c = mesh["coords"]
    f = lambda x, y: 3 * x ** 5 - 2 * x ** 2 * y ** 3 + y ** 4 + 0.5
    frames = np.zeros((1, 1, c.shape[0]))
    frames[0, 0] = f(c[:, 0], c[:, 1])
    g = pkg.wavefield.Grid(mesh, 17, 13, "bottom")
    P = g.points()
    img = g.interpolate(frames, [-1, -1, -1, -1, 0], 3, H)[0]
    g.close()
    exact = f(P["xp"], P["yp"]).reshape(17, 13).T
    assert np.abs(img - exact).max() <= 1e-12 * np.abs(exact).max()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_interpolation_from_plan_frames(pkg, precision):
    """All 15 frame fields recorded on the device, interpolated in place;
    compared with the oracle run's frames through the oracle interpolation."""
    from tests.test_flat_shell_gpu import oracle_run
    scs, run = pkg.workloads.plate_delamination(nex=8, ney=8, L=0.08, T=4e-5, f=200e3,
                                                zone=(0.04, 0.04, 0.02, 0.012, 0.3), layer=3, radius=0.03)
    sc = scs[0]
    run.nft = min(run.nft, 300)
    sc.signal = sc.signal[:run.nft]
    run.frm_int, run.frame_dof, run.frame_kind = 60, 0, 3
    plan = pkg.Plan(scs, run, precision=precision, path=0)
    res = plan.forward(want_frames=True)[0]
    _, ref = oracle_run(sc, run)
    assert res["frames"].shape == ref["frames"].shape == (run.nft // 60, 15, sc.mesh["coords"].shape[0])
    # FP32 state: 1e-3 on displacement/velocity, acceleration (a second
    # difference of the state) 1e-2
    tols = (1e-10,) * 3 if precision == 64 else (1e-3, 1e-3, 1e-2)
    for kind in range(3):
        sl = slice(5 * kind, 5 * kind + 5)
        assert rel(res["frames"][:, sl], ref["frames"][:, sl]) <= tols[kind], kind
    comps = ("x", "Fix", "y", "Fiy", "z")
    n = 20
    for surface in ("top", "bottom"):
        g = pkg.wavefield.Grid(sc.mesh, n, n, surface)
        for kind, fv in enumerate(("displacement", "velocity", "acceleration")):
            fields = {c: ref["frames"][:, 5 * kind + k] for k, c in enumerate(comps)}
            for motion in (3, 6, 9):
                got = g.from_plan(plan, motion, H, fv)
                want, _ = _oracle(sc.mesh, n, fields, motion, surface)
                assert rel(got, np.transpose(want, (2, 0, 1))) <= tols[kind], (surface, fv, motion)
        g.close()
    plan.close()


@pytest.mark.gpu
def test_reference_entry_points_write_frames_and_grid(pkg, tmp_path):
    """main_flat_shell writes the reference's frame files for field_variable
    'all' (15 per frame), spec2meshgrid_flat_shell reads them back and writes
    Data(Ny, Nx, nFrames); both match the oracle."""
    from scipy.io import loadmat
    M = pkg.materials
    mesh = pkg.mesh.structured_plate(0.06, 0.06, 6, 6)
    q = M.ply_stiffness(**M.CFRP_PLY)
    lam = M.laminate(q, M.CFRP_RHO, M.CFRP_PLY_T, M.CFRP_ANGLES)
    nft = 240
    dt = pkg.element.stable_dt([pkg.element.rect_nodes(0.01, 0.01)], [lam])
    inputs = dict(nft=nft, tt=dt * nft, f_1=50e3, f_2=250e3, t_1=0.0, nFrames=4, field_variable="all",
                  etad_xy=4e2, etad_z=4e3, V0=1.0, lh=np.array(M.CFRP_PLY_T), mat_table=M.table_row(lam))
    out = tmp_path / "out"
    tf = pkg.main_flat_shell(7, inputs, mesh, "gpu", str(out), precision=64)
    assert len(tf) == 4 and np.all(np.diff(tf) > 0)
    names = [p + c for p in "UVA" for c in ("x", "Fix", "y", "Fiy", "z")]
    for c in range(1, 5):
        for nm in names:
            v = loadmat(out / f"{nm}_frame{c}.mat")[nm]
            assert v.shape == (mesh["coords"].shape[0], 1)
    # oracle frames of the same run
    from oracle.oracle import OracleProblem
    orc = OracleProblem(mesh["nodes"], mesh["coords"], M.table_row(lam)[None, :])
    centre = pkg.mesh.nearest_node(mesh["coords"], 0.03, 0.03)
    _, st = pkg.hanning_signal(dt, nft, 50e3, 250e3, 0.0)
    ref = orc.run(dt, nft, st, nn_first=2, eta_xy=4e2, eta_z=4e3, force_dof=[5 * centre], force_val=[1.0],
                  out_dof=[5 * centre], h=float(np.sum(M.CFRP_PLY_T)), frm_int=nft // 4, frame_dof=0, frame_kind=3)
    for c in range(4):
        for k, nm in enumerate(names):
            got = loadmat(out / f"{nm}_frame{c + 1}.mat")[nm][:, 0]
            assert rel(got, ref["frames"][c, k]) <= 1e-10 or np.abs(ref["frames"][c, k]).max() == 0
    data = pkg.wavefield.spec2meshgrid_flat_shell(7, inputs, mesh, 16, 16, "velocity", 9, "top", str(out),
                                                  str(out))
    saved = loadmat(out / "flat_shell_total_velocities_7_16x16top.mat")["Data"]
    assert saved.shape == (16, 16, 4) and np.array_equal(saved, data)
    fields = {c: ref["frames"][:, 5 + k] for k, c in enumerate(("x", "Fix", "y", "Fiy", "z"))}
    want, _ = R.spec2meshgrid_flat_shell(mesh["nodes"], mesh["coords"], 16, 16, fields, 9, "top",
                                         float(np.sum(M.CFRP_PLY_T)))
    assert rel(data, want) <= 1e-10
