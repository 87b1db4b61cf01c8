"""shm_stiffness_static: the internal force for callers that cannot allocate.

Some callers of this library must not allocate device memory themselves: a
MATLAB MEX gateway whose gpuArray buffers belong to MATLAB's GPU memory
manager, or a monitoring loop that runs on a fixed memory budget and forbids
allocation after start-up.  For them the library offers one entry point that
allocates nothing and keeps its element-local forces in a fixed device array
inside the library.  These tests call it through the C ABI, on device buffers
that the test prepares, and compare it with the plan-based
shm_apply_stiffness within the FP64 tolerance used by the other tests:
two calls in a row (different displacements, separated by a synchronisation),
two calls queued back to back on one stream (the shared array is reused
without a host round trip), and a smaller mesh after a larger one (stale
element forces of the larger mesh must not leak into the smaller one).
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from oracle import ref_setup as R

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11


class StaticCase:
    """A distorted two-material mesh on the device, and a plan on the same
    mesh for the reference values."""

    def __init__(self, pkg, torch, nex, ney, seed):
        from tests.test_oracle_physics import _distorted, _materials
        mesh = _distorted(pkg, nex=nex, ney=ney, seed=seed)
        lams = _materials(pkg)
        table = np.stack([pkg.materials.table_row(l) for l in lams])
        self.fen = mesh["nodes"].shape[0]
        self.nnode = mesh["coords"].shape[0]
        em = np.arange(self.fen) % 2
        keep = np.linspace(0.4, 1.0, self.fen)
        IG, IL = R.nodes_maps_fiborek(mesh["nodes"], self.nnode, 5, 1)
        self.rows = IG.shape[0]
        sc = pkg.Scenario(mesh=mesh, mat_table=table, elem_mat=em, elem_keep=keep, signal=np.zeros(4))
        self.plan = pkg.Plan([sc], pkg.RunConfig(dt=1e-8, nft=4), precision=64, path=1)
        dev = torch.device("cuda:0")
        lam = (table[em][:, :21] * keep[:, None]).T.copy()  # [21 x fen]
        self.t = dict(
            nodes=torch.tensor(np.asarray(mesh["nodes"]).T.copy(), dtype=torch.int32, device=dev),
            coords=torch.tensor(np.asarray(mesh["coords"]).T.copy(), dtype=torch.float64, device=dev),
            lam=torch.tensor(lam, dtype=torch.float64, device=dev),
            ig=torch.tensor(IG.T.copy(), dtype=torch.int32, device=dev),
            il=torch.tensor(IL.T.copy(), dtype=torch.int32, device=dev))
        self.torch = torch

    def call(self, lib, t_U, t_F, stream, fen=None):
        t = self.t
        return lib.shm_stiffness_static(self.fen if fen is None else fen, self.nnode, t["nodes"].data_ptr(),
                                        t["coords"].data_ptr(), t["lam"].data_ptr(), self.rows, t["ig"].data_ptr(),
                                        t["il"].data_ptr(), t_U.data_ptr(), t_F.data_ptr(), stream)

    def check(self, F_static, U, what):
        F_plan = self.plan.apply_stiffness(U)
        err = np.linalg.norm(F_static - F_plan) / np.linalg.norm(F_plan)
        assert np.isfinite(err) and err <= FP64_TOL, (what, err)


def test_static_stiffness_matches_plan(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.native.load()
    big = StaticCase(pkg, torch, 6, 5, seed=7)
    small = StaticCase(pkg, torch, 3, 2, seed=8)
    dev = torch.device("cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(11)

    # two calls in a row, each waited for
    t_F = torch.zeros(5 * big.nnode, dtype=torch.float64, device=dev)
    for call in range(2):
        U = rng.standard_normal(5 * big.nnode) * 1e-9 * (call + 1)
        t_U = torch.tensor(U, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        assert big.call(lib, t_U, t_F, stream) == pkg.native.SHM_OK
        torch.cuda.synchronize()
        big.check(t_F.cpu().numpy(), U, f"call {call}")

    # two calls queued back to back on one stream, no synchronisation between
    Us = [rng.standard_normal(5 * big.nnode) * 1e-9 for _ in range(2)]
    t_Us = [torch.tensor(U, dtype=torch.float64, device=dev) for U in Us]
    t_Fs = [torch.full((5 * big.nnode,), np.nan, dtype=torch.float64, device=dev) for _ in range(2)]
    torch.cuda.synchronize()
    for t_U, t_F2 in zip(t_Us, t_Fs):
        assert big.call(lib, t_U, t_F2, stream) == pkg.native.SHM_OK
    torch.cuda.synchronize()
    for k in range(2):
        big.check(t_Fs[k].cpu().numpy(), Us[k], f"queued call {k}")

    # a smaller mesh after the larger one reuses the array's first slots only
    U = rng.standard_normal(5 * small.nnode) * 1e-9
    t_U = torch.tensor(U, dtype=torch.float64, device=dev)
    t_F = torch.zeros(5 * small.nnode, dtype=torch.float64, device=dev)
    assert small.call(lib, t_U, t_F, stream) == pkg.native.SHM_OK
    torch.cuda.synchronize()
    small.check(t_F.cpu().numpy(), U, "smaller mesh")

    # sizes beyond the fixed array are refused before any device work
    st = big.call(lib, t_Us[0], t_Fs[0], stream, fen=pkg.native.SHM_STATIC_MAX_ELEMS + 1)
    assert st == pkg.native.SHM_ERR_BAD_ARG
    assert b"SHM_STATIC_MAX_ELEMS" in lib.shm_last_error(None)
    big.plan.close()
    small.plan.close()
