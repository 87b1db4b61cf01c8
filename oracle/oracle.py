"""Oracle driver: builds ``sem_oracle.c`` and runs the FP64 reference restatement.

TEST INFRASTRUCTURE ONLY (tests/, __graft_entry__.smoke(), bench.py's CPU
baseline / reference arm).  Parity unpinned for the time loop (no reference
golden outputs exist); set-up constants are pinned in tests/golden/.  All set-up quantities are recomputed here from
the restated reference functions in ``ref_setup.py``; nothing is taken from
the product except the raw inputs (mesh arrays, material table, signal).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from . import ref_setup as R

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libsemoracle.so")
SRC = os.path.join(HERE, "sem_oracle.c")

I32P = C.POINTER(C.c_int32)
I64P = C.POINTER(C.c_int64)
F64P = C.POINTER(C.c_double)


class OracleArgs(C.Structure):
    _fields_ = [("fen", C.c_int32), ("nnode", C.c_int32), ("nodes", I32P),
                ("nnzx", C.c_int32), ("nnzy", C.c_int32),
                ("nx_row", I32P), ("nx_col", I32P), ("nx_val", F64P),
                ("ny_row", I32P), ("ny_col", I32P), ("ny_val", F64P),
                ("invJ11", F64P), ("invJ12", F64P), ("invJ21", F64P), ("invJ22", F64P), ("WWDetJ", F64P),
                ("coef", F64P), ("rows5", C.c_int32), ("IGd", I64P), ("ILd", I64P),
                ("mg", F64P), ("mg2", F64P), ("mg0", F64P), ("cg", F64P), ("a0", C.c_double), ("a1", C.c_double),
                ("nn_first", C.c_int32), ("nft", C.c_int32), ("st", F64P), ("Fa", F64P),
                ("nout", C.c_int32), ("out_dof", I32P), ("displ", F64P),
                ("nsens", C.c_int32), ("sens_ptr", I32P), ("sens_el", I32P),
                ("pzt_thickness", C.c_double), ("g33", C.c_double), ("e31", C.c_double), ("e32", C.c_double),
                ("h", C.c_double), ("voltage", F64P),
                ("frm_int", C.c_int32), ("frame_dof", C.c_int32), ("frame_kind", C.c_int32),
                ("nframes_max", C.c_int32),
                ("frames", F64P), ("t_frames_step", F64P), ("nthreads", C.c_int32),
                ("U", F64P), ("uold", F64P), ("frames_written", C.c_int32), ("diverged_at", C.c_int32),
                ("n_pf", C.c_int32), ("p_t1", F64P), ("p_nodal", F64P), ("p_dt", C.c_double)]


def build(force: bool = False) -> str:
    """gcc -O3 -fopenmp; -ffp-contract=off keeps x86 and Arm results identical."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, SRC, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stderr)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def _load():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.oracle_flat_shell_run.restype = C.c_int
        _lib.oracle_flat_shell_run.argtypes = [C.POINTER(OracleArgs)]
        _lib.oracle_flat_shell_apply_k.restype = C.c_int
        _lib.oracle_flat_shell_apply_k.argtypes = [C.POINTER(OracleArgs), F64P]
    return _lib


def _p(a, t=F64P):
    return None if a is None else a.ctypes.data_as(t)


class OracleProblem:
    """Reference-structured set-up of one plate (main_flat_shell.m:35-650)."""

    def __init__(self, nodes1, coords, mat_table, elem_mat=None, elem_keep=None, I_G=None, I_L=None):
        self.nodes = np.ascontiguousarray(nodes1, dtype=np.int32)
        self.coords = np.asarray(coords, float)
        fen, npe = self.nodes.shape
        assert npe == 36
        self.fen, self.nnode = fen, self.coords.shape[0]
        nx = ny = 6
        ksi, wx = R.gll(nx)
        eta, wy = R.gll(ny)
        Qx, Qy = R.vandermonde(ksi), R.vandermonde(eta)
        self.Nprimx, self.Nprimy = R.shape2d_prim(nx, ny, Qx, Qy, ksi, eta)
        self.px = R.sparse_pattern(self.Nprimx)
        self.py = R.sparse_pattern(self.Nprimy)
        jac = R.jacobians(self.nodes, self.coords, self.Nprimx, self.Nprimy)
        ww = R.quad_weights(nx, ny, wx, wy)
        self.WWDetJ = np.tile(ww, fen) * jac["detJ"]
        self.jac = jac
        tab = np.atleast_2d(np.asarray(mat_table, float))
        em = np.zeros(fen, np.int64) if elem_mat is None else np.asarray(elem_mat, np.int64)
        keep = np.ones(fen) if elem_keep is None else np.asarray(elem_keep, float)
        per_el = tab[em]                                          # [fen, 23]
        coef = per_el[:, :21] * keep[:, None]
        # per-local-node arrays as composite_plate_c_delam*.m produce them
        self.coef = np.ascontiguousarray(np.repeat(coef.T, 36, axis=1))   # [21, fen*36]
        self.m11 = np.repeat(per_el[:, 21], 36)
        self.I11 = np.repeat(per_el[:, 22], 36)
        if I_G is None:
            I_G, I_L = R.nodes_maps_fiborek(self.nodes, self.nnode, 5, 1)
        self.I_G, self.I_L = np.asarray(I_G, np.int64), np.asarray(I_L, np.int64)
        self.Gd, self.Ld = R.basket_dofs(self.I_G, self.I_L)
        self.ndof = 5 * self.nnode
        self.mg_raw = R.mass_vector(self.WWDetJ, self.m11, self.I11, self.Gd, self.Ld, self.ndof)

    def coefficients(self, dt, eta_xy, eta_z):
        """main_flat_shell.m:575-604."""
        a0 = 1 / dt ** 2
        a1 = 1 / (2 * dt)
        a2 = 2 * a0
        dv = np.zeros(self.ndof)
        dv[0::5] = eta_xy
        dv[2::5] = eta_xy
        dv[4::5] = eta_z
        mg = self.mg_raw
        cg = dv * mg
        mg2 = a2 * mg
        mgs = a0 * mg
        mg0 = 1.0 / (mgs + a1 * cg)
        return a0, a1, mgs, mg2, mg0, cg

    def _args(self, keep):
        px, py = self.px, self.py
        A = OracleArgs()
        A.fen, A.nnode = self.fen, self.nnode
        A.nodes = _p(self.nodes, I32P)
        A.nnzx, A.nnzy = len(px[0]), len(py[0])
        A.nx_row, A.nx_col, A.nx_val = _p(px[0], I32P), _p(px[1], I32P), _p(px[2])
        A.ny_row, A.ny_col, A.ny_val = _p(py[0], I32P), _p(py[1], I32P), _p(py[2])
        j = self.jac
        A.invJ11, A.invJ12 = _p(j["invJ11"]), _p(j["invJ12"])
        A.invJ21, A.invJ22 = _p(j["invJ21"]), _p(j["invJ22"])
        A.WWDetJ = _p(self.WWDetJ)
        A.coef = _p(self.coef)
        Gd = np.ascontiguousarray(self.Gd.T)   # column-major: basket-major rows
        Ld = np.ascontiguousarray(self.Ld.T)
        keep += [Gd, Ld]
        A.rows5 = self.Gd.shape[0]
        A.IGd, A.ILd = _p(Gd, I64P), _p(Ld, I64P)
        return A

    def apply_k(self, U):
        keep = []
        A = self._args(keep)
        U = np.ascontiguousarray(U, float).copy()
        F = np.zeros_like(U)
        A.U = _p(U)
        rc = _load().oracle_flat_shell_apply_k(C.byref(A), _p(F))
        assert rc == 0
        return F

    def run(self, dt, nft, st, nn_first=2, eta_xy=0.0, eta_z=0.0, force_dof=(), force_val=(), out_dof=(),
            sensors=(), pzt=None, h=0.0, frm_int=0, frame_dof=5, frame_kind=0, U0=None, uold0=None, nthreads=0,
            nn_last=None, pressure=None):
        keep = []
        A = self._args(keep)
        a0, a1, mgs, mg2, mg0, cg = self.coefficients(dt, eta_xy, eta_z)
        keep += [mgs, mg2, mg0, cg]
        A.mg, A.mg2, A.mg0, A.cg = _p(mgs), _p(mg2), _p(mg0), _p(cg)
        A.a0, A.a1 = a0, a1
        A.nn_first, A.nft = nn_first, (nft if nn_last is None else nn_last)
        st = np.ascontiguousarray(st, float)
        A.st = _p(st)
        Fa = np.zeros(self.ndof)
        for d, v in zip(force_dof, force_val):
            Fa[int(d) - 1] += v
        A.Fa = _p(Fa)
        od = np.ascontiguousarray(out_dof, np.int32)
        displ = np.zeros(max(len(od), 1) * nft)
        A.nout, A.out_dof, A.displ = len(od), _p(od, I32P), _p(displ)
        if sensors:
            ptr = np.zeros(len(sensors) + 1, np.int32)
            ptr[1:] = np.cumsum([len(s) for s in sensors])
            els = np.concatenate([np.asarray(s, np.int32) for s in sensors])
            keep += [ptr, els]
            A.nsens, A.sens_ptr, A.sens_el = len(sensors), _p(ptr, I32P), _p(els, I32P)
            A.pzt_thickness, A.g33, A.e31, A.e32 = pzt["pzt_thickness"], pzt["g33"], pzt["e31"], pzt["e32"]
        else:
            A.nsens = 0
        A.h = h
        voltage = np.zeros(max(len(sensors), 1) * nft)
        A.voltage = _p(voltage)
        # frames at every nn in [nn_first, nft] with nn % frm_int == 0
        nfr = (nft // frm_int - (nn_first + frm_int - 1) // frm_int + 1) if frm_int else 0
        nfld = (3 if frame_kind == 3 else 1) * (5 if frame_dof == 0 else 1)
        frames = np.zeros(max(nfr * nfld, 1) * self.nnode)
        tfs = np.zeros(max(nfr, 1))
        A.frm_int, A.frame_dof, A.frame_kind, A.nframes_max = frm_int, frame_dof, frame_kind, nfr
        A.frames, A.t_frames_step = _p(frames), _p(tfs)
        A.nthreads = nthreads
        if pressure is not None:  # dict(times=[npf], nodal=[npf, nnode]); t_sem = (nn-1)*dt
            pt1 = np.ascontiguousarray(pressure["times"], float)
            pnod = np.ascontiguousarray(pressure["nodal"], float).reshape(len(pt1), self.nnode)
            keep += [pt1, pnod]
            A.n_pf, A.p_t1, A.p_nodal, A.p_dt = len(pt1), _p(pt1), _p(pnod), dt
        else:
            A.n_pf = 0
        U = np.zeros(self.ndof) if U0 is None else np.ascontiguousarray(U0, float).copy()
        Uo = np.zeros(self.ndof) if uold0 is None else np.ascontiguousarray(uold0, float).copy()
        A.U, A.uold = _p(U), _p(Uo)
        rc = _load().oracle_flat_shell_run(C.byref(A))
        assert rc == 0
        return dict(displ=displ[:len(od) * nft].reshape(nft, len(od)) if len(od) else np.zeros((nft, 0)),
                    voltage=voltage[:len(sensors) * nft].reshape(nft, len(sensors)) if sensors else np.zeros((nft, 0)),
                    frames=frames[:nfr * nfld * self.nnode].reshape(nfr, nfld, self.nnode), U=U, uold=Uo,
                    diverged_at=A.diverged_at, frames_written=A.frames_written)


class OracleSolidArgs(C.Structure):
    _fields_ = [("fen", C.c_int32), ("nnode", C.c_int32), ("nodes", I32P), ("nnz", C.c_int32 * 3),
                ("row", I32P * 3), ("col", I32P * 3), ("val", F64P * 3), ("invJ", F64P), ("W", F64P),
                ("D", F64P), ("rows3", C.c_int32), ("IGd", I64P), ("ILd", I64P),
                ("mg", F64P), ("mg2", F64P), ("mg0", F64P), ("cg", F64P), ("a0", C.c_double), ("a1", C.c_double),
                ("nn_first", C.c_int32), ("nft", C.c_int32), ("st", F64P), ("Fa", F64P),
                ("nout", C.c_int32), ("out_dof", I32P), ("displ", F64P), ("nthreads", C.c_int32),
                ("U", F64P), ("uold", F64P)]


class OracleSolid:
    """Reference-structured set-up of a 3D solid plate (main_spec3Dcuda_global_...)."""

    def __init__(self, nodes1, coords, dtable, rho, elem_mat=None, elem_keep=None):
        self.nodes = np.ascontiguousarray(nodes1, dtype=np.int32)
        self.coords = np.asarray(coords, float)
        fen, npe = self.nodes.shape
        assert npe == 108
        self.fen, self.nnode = fen, self.coords.shape[0]
        Nx, Ny, Nz = R.shape3d_blocks()
        self.pat = [R.sparse_pattern(N) for N in (Nx, Ny, Nz)]
        self.invJ, self.W = R.jacobians3d(self.nodes, self.coords, Nx, Ny, Nz)
        em = np.zeros(fen, np.int64) if elem_mat is None else np.asarray(elem_mat, np.int64)
        keep = np.ones(fen) if elem_keep is None else np.asarray(elem_keep, float)
        dt_ = np.atleast_2d(np.asarray(dtable, float))[em] * keep[:, None]          # [fen, 13]
        self.D = np.ascontiguousarray(np.repeat(dt_.T, 108, axis=1))               # [13, fen*108]
        rho_e = np.asarray(rho, float)[em] if np.ndim(rho) else np.full(fen, float(rho))
        I_G, I_L = R.nodes_maps_fiborek(self.nodes, self.nnode, 5, 3)
        self.Gd, self.Ld = R.basket_dofs(I_G, I_L, 3)
        self.ndof = 3 * self.nnode
        mgL = np.repeat(self.W * np.repeat(rho_e, 108), 3)                           # mass3D_v2.m
        self.mg_raw = R.basket_scatter(mgL, self.Gd, self.Ld, self.ndof)

    def apply_k(self, U):
        """K U (3 DOF per node, reference DOF order) from one undamped,
        unforced step of the loop started at u_n = u_{n-1} = U: the update gives
        u_{n+1} = U - F / (a0 m), so F = a0 m (U - u_{n+1}); dt = 1 keeps the
        step's force term dominant (no cancellation in U - u_{n+1})."""
        U = np.asarray(U, float)
        r = self.run(1.0, 2, np.zeros(2), nn_first=2, U0=U, uold0=U)
        return self.mg_raw * (U - r["U"])

    def run(self, dt, nft, st, nn_first=2, eta_xy=0.0, eta_z=0.0, force_dof=(), force_val=(), out_dof=(),
            nthreads=0, U0=None, uold0=None):
        a0, a1 = 1 / dt ** 2, 1 / (2 * dt)
        dv = np.zeros(self.ndof)
        dv[0::3] = eta_xy
        dv[1::3] = eta_xy
        dv[2::3] = eta_z
        mg = self.mg_raw
        cg = dv * mg
        mg2 = 2 * a0 * mg
        mgs = a0 * mg
        mg0 = 1.0 / (mgs + a1 * cg)
        A = OracleSolidArgs()
        keep = [mg2, mgs, mg0, cg]
        A.fen, A.nnode = self.fen, self.nnode
        A.nodes = _p(self.nodes, I32P)
        for k in range(3):
            r, c_, v = self.pat[k]
            A.nnz[k] = len(r)
            A.row[k], A.col[k], A.val[k] = _p(r, I32P), _p(c_, I32P), _p(v)
        A.invJ, A.W, A.D = _p(self.invJ), _p(self.W), _p(self.D)
        Gd = np.ascontiguousarray(self.Gd.T)
        Ld = np.ascontiguousarray(self.Ld.T)
        keep += [Gd, Ld]
        A.rows3 = self.Gd.shape[0]
        A.IGd, A.ILd = _p(Gd, I64P), _p(Ld, I64P)
        A.mg, A.mg2, A.mg0, A.cg = _p(mgs), _p(mg2), _p(mg0), _p(cg)
        A.a0, A.a1 = a0, a1
        A.nn_first, A.nft = nn_first, nft
        st = np.ascontiguousarray(st, float)
        A.st = _p(st)
        Fa = np.zeros(self.ndof)
        for d, v in zip(force_dof, force_val):
            Fa[int(d) - 1] += v
        A.Fa = _p(Fa)
        od = np.ascontiguousarray(out_dof, np.int32)
        displ = np.zeros(max(len(od), 1) * nft)
        A.nout, A.out_dof, A.displ = len(od), _p(od, I32P), _p(displ)
        A.nthreads = nthreads
        U = np.zeros(self.ndof) if U0 is None else np.array(U0, float)
        Uo = np.zeros(self.ndof) if uold0 is None else np.array(uold0, float)
        A.U, A.uold = _p(U), _p(Uo)
        lib = _load()
        lib.oracle_solid_run.restype = C.c_int
        lib.oracle_solid_run.argtypes = [C.POINTER(OracleSolidArgs)]
        assert lib.oracle_solid_run(C.byref(A)) == 0
        return dict(displ=displ[:len(od) * nft].reshape(nft, len(od)), U=U, uold=Uo, mass=self.mg_raw)
