"""shm_stiffness_static: the internal force for callers that cannot allocate.

Some callers of this library must not allocate device memory themselves: a
MATLAB MEX gateway whose gpuArray buffers belong to MATLAB's GPU memory
manager, or a monitoring loop that runs on a fixed memory budget and forbids
allocation after start-up.  For them the library offers one entry point that
allocates nothing and keeps its element-local forces in a fixed device array
inside the library.  This test calls it through the C ABI, on device buffers
that the test prepares, and checks that two calls in a row (with different
displacements) give the same internal force as the plan-based
shm_apply_stiffness, within the FP64 tolerance used by the other tests.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from oracle import ref_setup as R

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11


def test_static_stiffness_matches_plan(pkg):
    torch = pytest.importorskip("torch")
    from tests.test_oracle_physics import _distorted, _materials
    mesh = _distorted(pkg, nex=6, ney=5, seed=7)
    lams = _materials(pkg)
    table = np.stack([pkg.materials.table_row(l) for l in lams])
    fen = mesh["nodes"].shape[0]
    nnode = mesh["coords"].shape[0]
    em = np.arange(fen) % 2
    keep = np.linspace(0.4, 1.0, fen)
    IG, IL = R.nodes_maps_fiborek(mesh["nodes"], nnode, 5, 1)

    # existing entry point: plan-based K*U (host arrays)
    sc = pkg.Scenario(mesh=mesh, mat_table=table, elem_mat=em, elem_keep=keep, signal=np.zeros(4))
    plan = pkg.Plan([sc], pkg.RunConfig(dt=1e-8, nft=4), precision=64, path=1)

    dev = torch.device("cuda:0")
    lam = (table[em][:, :21] * keep[:, None]).T.copy()  # [21 x fen]
    t_nodes = torch.tensor(np.asarray(mesh["nodes"]).T.copy(), dtype=torch.int32, device=dev)
    t_coords = torch.tensor(np.asarray(mesh["coords"]).T.copy(), dtype=torch.float64, device=dev)
    t_lam = torch.tensor(lam, dtype=torch.float64, device=dev)
    t_ig = torch.tensor(IG.T.copy(), dtype=torch.int32, device=dev)
    t_il = torch.tensor(IL.T.copy(), dtype=torch.int32, device=dev)
    t_F = torch.zeros(5 * nnode, dtype=torch.float64, device=dev)
    lib = pkg.native.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(11)
    for call in range(2):
        U = rng.standard_normal(5 * nnode) * 1e-9 * (call + 1)
        t_U = torch.tensor(U, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = lib.shm_stiffness_static(fen, nnode, t_nodes.data_ptr(), t_coords.data_ptr(), t_lam.data_ptr(),
                                      IG.shape[0], t_ig.data_ptr(), t_il.data_ptr(), t_U.data_ptr(),
                                      t_F.data_ptr(), stream)
        assert st == pkg.native.SHM_OK
        torch.cuda.synchronize()
        F_static = t_F.cpu().numpy()
        F_plan = plan.apply_stiffness(U)
        err = np.linalg.norm(F_static - F_plan) / np.linalg.norm(F_plan)
        assert np.isfinite(err) and err <= FP64_TOL, (call, err)
    plan.close()

    # sizes beyond the fixed array are refused before any device work
    big = pkg.native.SHM_ERR_BAD_ARG
    st = lib.shm_stiffness_static(4097, nnode, t_nodes.data_ptr(), t_coords.data_ptr(), t_lam.data_ptr(),
                                  IG.shape[0], t_ig.data_ptr(), t_il.data_ptr(), t_F.data_ptr(), t_F.data_ptr(),
                                  stream)
    assert st == big
