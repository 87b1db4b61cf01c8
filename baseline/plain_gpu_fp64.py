"""Reference-structured FP64 GPU loop (measurement baseline, not the product).

The reference's GPU path is MATLAB ``gpuArray`` vectorisation of the MAIN LOOP
(src/models/flat_shell/flat_shell_engine/main_flat_shell.m:651-750): indexed
gathers, sparse block-diagonal derivative operators Npx/Npy (:661-671), the
resultant expressions over all local nodes (:674-681), 20 transposed sparse
products (:683-689), the 12-basket scatter (:724-726) and the update
(:742-750), every one a separate device operation.  MATLAB is not available,
so this module issues the same sequence of operations with PyTorch in FP64
(cuSPARSE CSR SpMV, gathers, element-wise kernels, index_add).  It is the
"plain single-scenario FP64 GPU path" that the batched FP32 engine is
compared against; its outputs are checked against the engine's FP64 path.
"""
from __future__ import annotations

import numpy as np
import torch


def _block_csr(D: np.ndarray, fen: int, along_xi: bool, device):
    """Npx = I (x) D (xi) or Npy = D (x) I (eta) per element, block diagonal."""
    n = D.shape[0]
    B = np.kron(np.eye(n), D) if along_xi else np.kron(D, np.eye(n))
    r, c = np.nonzero(B)
    v = B[r, c]
    nb = n * n
    rows = (np.arange(fen)[:, None] * nb + r[None, :]).reshape(-1)
    cols = (np.arange(fen)[:, None] * nb + c[None, :]).reshape(-1)
    vals = np.tile(v, fen)
    L = fen * nb
    coo = torch.sparse_coo_tensor(torch.tensor(np.stack([rows, cols])), torch.tensor(vals), (L, L),
                                  dtype=torch.float64, device=device)
    return coo.coalesce().to_sparse_csr(), coo.transpose(0, 1).coalesce().to_sparse_csr()


class PlainFP64:
    def __init__(self, pkg, sc, run, device="cuda"):
        dev = torch.device(device)
        self.dev = dev
        nodes = np.asarray(sc.mesh["nodes"])
        coords = np.asarray(sc.mesh["coords"])
        fen = nodes.shape[0]
        nnode = coords.shape[0]
        self.ndof = 5 * nnode
        _, w, D = pkg.element.gll_derivative_matrix(6)
        self.Npx, self.Npxt = _block_csr(D, fen, True, dev)
        self.Npy, self.Npyt = _block_csr(D, fen, False, dev)
        I = torch.tensor(nodes.reshape(-1) - 1, device=dev, dtype=torch.int64)
        self.Iu, self.Ifix, self.Iv, self.Ifiy, self.Iw = (5 * I + k for k in range(5))
        X = torch.tensor(coords[:, 0], device=dev)[I]
        Y = torch.tensor(coords[:, 1], device=dev)[I]
        J11 = self.Npx @ X
        J21 = self.Npx @ Y
        J12 = self.Npy @ X
        J22 = self.Npy @ Y
        a = 1.0 / (J11 * J22 - J12 * J21)
        self.i11, self.i12, self.i21, self.i22 = a * J22, -a * J12, -a * J21, a * J11
        ww = torch.tensor(np.outer(w, w).reshape(-1), device=dev)
        self.W = ww.repeat(fen) * (J11 * J22 - J12 * J21)
        tab = np.atleast_2d(sc.mat_table)
        em = np.zeros(fen, int) if sc.elem_mat is None else np.asarray(sc.elem_mat)
        keep = np.ones(fen) if sc.elem_keep is None else np.asarray(sc.elem_keep)
        per = tab[em][:, :21] * keep[:, None]
        self.c = [torch.tensor(np.repeat(per[:, k], 36), device=dev) for k in range(21)]
        # mass by the 12-basket scatter of WWDetJ * [m11, I11, m11, I11, m11]
        m11 = torch.tensor(np.repeat(tab[em][:, 21], 36), device=dev)
        I11 = torch.tensor(np.repeat(tab[em][:, 22], 36), device=dev)
        L = fen * 36
        mgL = torch.zeros(5 * L, device=dev, dtype=torch.float64)
        mgL[0::5], mgL[1::5], mgL[2::5], mgL[3::5], mgL[4::5] = (self.W * m11, self.W * I11, self.W * m11,
                                                                  self.W * I11, self.W * m11)
        # baskets: local copies of each global DOF, 12 conflict-free groups
        g = (5 * I[:, None] + torch.arange(5, device=dev)[None, :]).reshape(-1)
        order = torch.argsort(g, stable=True)
        gs = g[order]
        first = torch.ones_like(gs, dtype=torch.bool)
        first[1:] = gs[1:] != gs[:-1]
        rank = torch.arange(len(gs), device=dev) - torch.cummax(torch.where(first, torch.arange(len(gs), device=dev),
                                                                            torch.zeros_like(gs)), 0)[0]
        self.baskets = [(gs[rank == b], order[rank == b]) for b in range(int(rank.max()) + 1)]
        mg = torch.zeros(self.ndof, device=dev, dtype=torch.float64)
        for G_, L_ in self.baskets:
            mg.index_add_(0, G_, mgL[L_])
        dt = run.dt
        a0, a1 = 1 / dt ** 2, 1 / (2 * dt)
        dv = torch.zeros(self.ndof, device=dev, dtype=torch.float64)
        dv[0::5], dv[2::5], dv[4::5] = run.eta_xy, run.eta_xy, run.eta_z
        cg = dv * mg
        self.mg2, self.mg, self.mg0, self.a1cg = 2 * a0 * mg, a0 * mg, 1.0 / (a0 * mg + a1 * cg), a1 * cg
        self.Fa = torch.zeros(self.ndof, device=dev, dtype=torch.float64)
        self.Fa[torch.tensor(np.asarray(sc.force_dof) - 1, device=dev)] = torch.tensor(np.asarray(sc.force_val, float),
                                                                                      device=dev)
        self.st = torch.tensor(np.asarray(sc.signal, float), device=dev)
        self.out = torch.tensor(np.asarray(sc.out_dof) - 1, device=dev)
        self.U = torch.zeros(self.ndof, device=dev, dtype=torch.float64)
        self.uold = torch.zeros_like(self.U)
        self.F2 = torch.zeros(5 * L, device=dev, dtype=torch.float64)
        self.nn = run.nn_first
        self.displ = []

    def step(self):
        U = self.U
        UX, UY, UZ, FIX, FIY = U[self.Iu], U[self.Iv], U[self.Iw], U[self.Ifix], U[self.Ifiy]
        Npx, Npy = self.Npx, self.Npy
        NpxUX, NpxUY, NpxFIX, NpxFIY = Npx @ UX, Npx @ UY, Npx @ FIX, Npx @ FIY
        NpyUX, NpyUY, NpyFIX, NpyFIY = Npy @ UX, Npy @ UY, Npy @ FIX, Npy @ FIY
        NpxUZ, NpyUZ = Npx @ UZ, Npy @ UZ
        i11, i12, i21, i22 = self.i11, self.i12, self.i21, self.i22
        (a11, a12, a16, a22, a26, a66, a44, a45, a55, b11, b12, b16, b22, b26, b66,
         d11, d12, d16, d22, d26, d66) = self.c
        ex, exy_u = NpxUX * i11 + NpyUX * i21, NpxUX * i12 + NpyUX * i22
        kx, kxy_f = NpxFIX * i11 + NpyFIX * i21, NpxFIX * i12 + NpyFIX * i22
        ey, eyx_v = NpxUY * i12 + NpyUY * i22, NpxUY * i11 + NpyUY * i21
        ky, kyx_f = NpxFIY * i12 + NpyFIY * i22, NpxFIY * i11 + NpyFIY * i21
        Sxx = ex * a11 + kx * b11 + ey * a12 + ky * b12 + exy_u * a16 + kxy_f * b16 + eyx_v * a16 + kyx_f * b16
        Sxxz = ex * b11 + kx * d11 + ey * b12 + ky * d12 + exy_u * b16 + kxy_f * d16 + eyx_v * b16 + kyx_f * d16
        Sxy = ex * a16 + kx * b16 + ey * a26 + ky * b26 + exy_u * a66 + kxy_f * b66 + eyx_v * a66 + kyx_f * b66
        Sxyz = ex * b16 + kx * d16 + ey * b26 + ky * d26 + exy_u * b66 + kxy_f * d66 + eyx_v * b66 + kyx_f * d66
        Syy = ex * a12 + kx * b12 + ey * a22 + ky * b22 + exy_u * a26 + kxy_f * b26 + eyx_v * a26 + kyx_f * b26
        Syyz = ex * b12 + kx * d12 + ey * b22 + ky * d22 + exy_u * b26 + kxy_f * d26 + eyx_v * b26 + kyx_f * d26
        gy = FIY + NpxUZ * i12 + NpyUZ * i22
        gx = FIX + NpxUZ * i11 + NpyUZ * i21
        Syz = gy * a44 + gx * a45
        Sxz = gy * a45 + gx * a55
        W = self.W
        Xt, Yt = self.Npxt, self.Npyt
        fu = Xt @ (Sxx * i11 * W) + Yt @ (Sxx * i21 * W) + Xt @ (Sxy * i12 * W) + Yt @ (Sxy * i22 * W)
        fv = Xt @ (Syy * i12 * W) + Yt @ (Syy * i22 * W) + Xt @ (Sxy * i11 * W) + Yt @ (Sxy * i21 * W)
        mx = Xt @ (Sxxz * i11 * W) + Yt @ (Sxxz * i21 * W) + Xt @ (Sxyz * i12 * W) + Yt @ (Sxyz * i22 * W) + Sxz * W
        my = Xt @ (Syyz * i12 * W) + Yt @ (Syyz * i22 * W) + Xt @ (Sxyz * i11 * W) + Yt @ (Sxyz * i21 * W) + Syz * W
        fw = Xt @ (Syz * i12 * W) + Yt @ (Syz * i22 * W) + Xt @ (Sxz * i11 * W) + Yt @ (Sxz * i21 * W)
        F2 = self.F2
        F2[0::5], F2[1::5], F2[2::5], F2[3::5], F2[4::5] = fu, mx, fv, my, fw
        F = torch.zeros(self.ndof, device=self.dev, dtype=torch.float64)
        for G_, L_ in self.baskets:
            F.index_add_(0, G_, F2[L_])
        F = -F + self.mg2 * U + self.Fa * self.st[self.nn - 1] - self.mg * self.uold + self.a1cg * self.uold
        unew = self.mg0 * F
        self.displ.append(U[self.out])
        self.uold, self.U = U, unew
        self.nn += 1


def rate(pkg, sc, run, steps=50, warmup=5):
    """DOF-steps/s of the plain FP64 loop (CUDA events) and its first outputs."""
    p = PlainFP64(pkg, sc, run)
    for _ in range(warmup):
        p.step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        p.step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    displ = torch.stack(p.displ).cpu().numpy()
    return p.ndof * steps / (ms / 1e3), displ
