"""The reference's solver entry points end to end: arguments as the MATLAB
functions take them, files written as the MATLAB functions write them
(scipy.io .mat), read back and compared with the FP64 oracle.

* main_flat_shell_multi_pzt_c (main_flat_shell_multi_pzt_c.m:1): three
  bonded PZTs, the second driven, every PZT a sensor -> voltage<N>.mat
  [nft x 3] (:721), displ<N>.mat (w at the plate centre, :719), time<N>.mat
  with TotalNofNodes = dof/5 (:860-861), velocity frames (:696-835).
* main_flat_shell with a PZT in the mesh (main_flat_shell.m:121-225): the
  first PZT is actuator and sensor -> voltage<N>.mat (:925) and
  TotalNofNodes = dof/3 as that file computes it (:929)."""
import numpy as np
import pytest

from oracle.oracle import OracleProblem

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def _inputs(pkg, dt, nft, nframes, f):
    M = pkg.materials
    q = M.ply_stiffness(**M.CFRP_PLY)
    p = M.pzt5a()
    return dict(nft=nft, tt=dt * (nft - 1), f_1=f / 5, f_2=f, t_1=0.0, nFrames=nframes,
                field_variable="velocity", etad_xy=4e2, etad_z=4e3, V0=100.0, rho=M.CFRP_RHO,
                lh=np.array(M.CFRP_PLY_T), lalpha=np.array(M.CFRP_ANGLES), Spzt=p["S"], dp=p["d"], epsT=p["epsT"],
                theta_pzt=0.0, rho_pzt=p["rho"], pzt_thickness=0.2e-3, **q)


def _oracle(sc, run):
    orc = OracleProblem(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table, sc.elem_mat, sc.elem_keep)
    return orc.run(run.dt, run.nft, sc.signal, nn_first=run.nn_first, eta_xy=run.eta_xy, eta_z=run.eta_z,
                   force_dof=sc.force_dof, force_val=sc.force_val, out_dof=sc.out_dof,
                   sensors=[np.asarray(s) for s in sc.sensors], pzt=sc.pzt, h=run.h, frm_int=run.frm_int,
                   frame_dof=run.frame_dof, frame_kind=run.frame_kind)


def test_multi_pzt_entry_point_writes_reference_files(pkg, tmp_path):
    from scipy.io import loadmat
    nft, f = 200, 150e3
    scs, run = pkg.workloads.plate_multi_pzt(nex=16, L=0.08, nft=nft, actuator_no=2, f=f)
    sc = scs[0]
    mesh = dict(sc.mesh)
    mesh["pztEl"] = [np.asarray(e) + 1 for e in sc.sensors]   # MATLAB cell array of 1-based elements
    inputs = _inputs(pkg, run.dt, nft, 4, f)
    out = tmp_path / "multi"
    tf = pkg.main_flat_shell_multi_pzt_c(2, 5, inputs, mesh, "gpu", str(out), precision=64)
    # the same run through the oracle: frames of all five velocity fields every nft/4 steps
    run.frm_int, run.frame_dof, run.frame_kind = nft // 4, 0, 0
    ref = _oracle(sc, run)
    volt = loadmat(out / "voltage5.mat")["voltage"]
    displ = loadmat(out / "displ5.mat")["displ"]
    tinfo = loadmat(out / "time5.mat")
    assert volt.shape == (nft, 3) and displ.shape == (nft, 1)
    assert np.all(np.abs(ref["voltage"]).max(axis=0) > 0)
    assert rel(volt, ref["voltage"]) <= FP64_TOL
    assert rel(displ, ref["displ"]) <= FP64_TOL
    assert np.asarray(tinfo["TotalNofNodes"]).item() == mesh["coords"].shape[0]          # dof/5
    assert tinfo["t"].size == nft and np.asarray(tinfo["averageTime"]).item() > 0
    assert len(tf) == 4 and np.allclose(tf, (np.arange(1, 5) * (nft // 4) - 1) * inputs["tt"] / (nft - 1))
    for c in range(4):
        for k, nm in enumerate(("Vx", "VFix", "Vy", "VFiy", "Vz")):
            got = loadmat(out / f"{nm}_frame{c + 1}.mat")[nm][:, 0]
            want = ref["frames"][c, k]
            assert np.abs(want).max() == 0 or rel(got, want) <= FP64_TOL, (c, nm)
    with pytest.raises(ValueError):
        pkg.main_flat_shell_multi_pzt_c(4, 5, inputs, mesh, "gpu", str(out))
    with pytest.raises(ValueError):
        pkg.main_flat_shell_multi_pzt_c(1, 5, inputs, mesh, "cpu", str(out))


def test_main_flat_shell_with_pzt_writes_voltage(pkg, tmp_path):
    from scipy.io import loadmat
    nft, f = 160, 150e3
    scs, run = pkg.workloads.plate_multi_pzt(nex=12, L=0.06, n_pzt=1, actuator_no=1, nft=nft, f=f)
    sc = scs[0]
    mesh = dict(sc.mesh)
    mesh["pztEl"] = (np.asarray(sc.sensors[0]) + 1)[None, :]    # one PZT per row
    inputs = _inputs(pkg, run.dt, nft, 0, f)
    inputs["tt"] = run.dt * nft                                 # main_flat_shell.m: dt = tt/nft
    out = tmp_path / "single"
    pkg.main_flat_shell(3, inputs, mesh, "gpu", str(out), precision=64)
    run.nn_first = 2
    centre = pkg.mesh.nearest_node(mesh["coords"], 0.03, 0.03)
    sc.out_dof = np.array([5 * centre], np.int32)
    ref = _oracle(sc, run)
    volt = loadmat(out / "voltage3.mat")["voltage"]
    assert volt.shape == (nft, 1) and np.abs(ref["voltage"]).max() > 0
    assert rel(volt, ref["voltage"]) <= FP64_TOL
    assert rel(loadmat(out / "displ3.mat")["displ"], ref["displ"]) <= FP64_TOL
    assert np.asarray(loadmat(out / "time3.mat")["TotalNofNodes"]).item() == 5 * mesh["coords"].shape[0] / 3
