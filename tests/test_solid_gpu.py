"""3D solid plate (6x6x3 hexahedra) through the C ABI against the FP64 oracle's
restatement of main_spec3Dcuda_global_..._mat.m, with and without a
delamination (split interface nodes)."""
import numpy as np
import pytest

from oracle.oracle import OracleSolid

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def small_solid(pkg, delam):
    scs, run = pkg.workloads.solid_plate(nex=4, L=0.02, T=6e-6, f=800e3, n_out=4, radius=0.006, delam=False)
    sc = scs[0]
    if delam:
        sc.mesh = pkg.mesh.split_interface(sc.mesh, 3, [5, 6, 9, 10])
    run.nft = min(run.nft, 220)
    sc.signal = sc.signal[:run.nft]
    sc.elem_keep = np.linspace(0.6, 1.0, sc.mesh["nodes"].shape[0])
    return sc, run


@pytest.mark.parametrize("delam", [False, True])
def test_solid_matches_oracle(pkg, delam):
    sc, run = small_solid(pkg, delam)
    orc = OracleSolid(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table[:, :13], sc.mat_table[:, 13], sc.elem_mat,
                      sc.elem_keep)
    ref = orc.run(run.dt, run.nft, sc.signal, nn_first=run.nn_first, eta_xy=run.eta_xy, eta_z=run.eta_z,
                  force_dof=sc.force_dof, force_val=sc.force_val, out_dof=sc.out_dof)
    assert np.abs(ref["displ"]).max() > 0
    plan = pkg.SolidPlan([sc], run, precision=64, steps_per_graph=32)
    np.testing.assert_allclose(plan.mass(), ref["mass"], rtol=1e-12)
    got = plan.forward()[0]
    U, _ = plan.get_state()
    plan.close()
    assert rel(got["displ"], ref["displ"]) <= 1e-10
    assert rel(U, ref["U"]) <= 1e-10
    plan = pkg.SolidPlan([sc], run, precision=32)
    got32 = plan.forward()[0]
    plan.close()
    assert rel(got32["displ"], ref["displ"]) <= 1e-3


def test_solid_delamination_changes_response(pkg):
    a, run = small_solid(pkg, False)
    b, _ = small_solid(pkg, True)
    out = []
    for sc in (a, b):
        p = pkg.SolidPlan([sc], run, precision=64)
        out.append(p.forward()[0]["displ"])
        p.close()
    assert rel(out[1], out[0]) > 1e-6


def test_distorted_solid_uses_general_geometry(pkg):
    """In-plane jittered node columns make the hexahedra non-boxes: the kernel
    reads the per-node inverse Jacobians (the box path is for axis-aligned
    elements only); both agree with the oracle."""
    sc, run = small_solid(pkg, False)
    c = sc.mesh["coords"].copy()
    rng = np.random.default_rng(9)
    base = sc.mesh["base"]["coords"]
    L = base[:, 0].max()
    inner = (base[:, 0] > 0) & (base[:, 0] < L) & (base[:, 1] > 0) & (base[:, 1] < L)
    jit = np.zeros((base.shape[0], 2))
    jit[inner] = rng.uniform(-0.04, 0.04, (inner.sum(), 2)) * (L / 4 / 5)
    nxy = base.shape[0]
    for k in range(c.shape[0] // nxy):
        c[k * nxy:(k + 1) * nxy, :2] += jit
    sc.mesh = {**sc.mesh, "coords": c}
    orc = OracleSolid(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table[:, :13], sc.mat_table[:, 13], sc.elem_mat,
                      sc.elem_keep)
    ref = orc.run(run.dt, run.nft, sc.signal, nn_first=run.nn_first, eta_xy=run.eta_xy, eta_z=run.eta_z,
                  force_dof=sc.force_dof, force_val=sc.force_val, out_dof=sc.out_dof)
    plan = pkg.SolidPlan([sc], run, precision=64)
    got = plan.forward()[0]
    plan.close()
    assert np.abs(ref["displ"]).max() > 0
    assert rel(got["displ"], ref["displ"]) <= 1e-10
