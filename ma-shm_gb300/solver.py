"""Host side of the engine: plans, scenarios and the reference's solver entry point.

``main_flat_shell`` and ``main_flat_shell_multi_pzt_c`` mirror the reference's
``t_frames = main_flat_shell(test_case, input_no, meshfile, mode, output_name, tasks)``
(src/models/flat_shell/flat_shell_engine/main_flat_shell.m:1) and
``main_flat_shell_multi_pzt_c(actuator_no, ...)`` (main_flat_shell_multi_pzt_c.m:1)
with their output layout (displ<N>.mat, voltage<N>.mat for PZT plates,
time<N>.mat, {U,V,A}?_frame<c>.mat).  The time
loop itself runs in libshmsem.so on the GPU; this module only prepares inputs
and writes results.  There is no CPU path: ``mode`` other than 'gpu' raises.
"""
from __future__ import annotations

import ctypes as C
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import native
from .materials import table_row

FIELD_NAMES = ("x", "Fix", "y", "Fiy", "z")  # DOF order u, phi_x, v, phi_y, w


@dataclass
class Scenario:
    """One plate: mesh, laminate per element, excitation and outputs."""
    mesh: dict                       # nodes [fen,36] 1-based, coords [nnode,3], optional nex/ney, I_G/I_L
    mat_table: np.ndarray            # [nmat, 23]
    elem_mat: np.ndarray | None = None
    elem_keep: np.ndarray | None = None
    force_dof: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))   # 1-based DOF
    force_val: np.ndarray = field(default_factory=lambda: np.zeros(0))
    out_dof: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))     # 1-based DOF
    sensors: list = field(default_factory=list)   # list of 0-based element arrays (PZT sensors)
    pzt: dict | None = None          # pzt_thickness, g33, e31, e32
    signal: np.ndarray | None = None  # st [nft]
    pressure: dict | None = None     # times [npf] (s), nodal [npf, nnode] (Pa): pressure loading


@dataclass
class RunConfig:
    dt: float
    nft: int
    nn_first: int = 2
    eta_xy: float = 0.0
    eta_z: float = 0.0
    h: float = 0.0
    frm_int: int = 0
    frame_dof: int = 5               # 0 = all five components, else 1..5 (5 = w)
    frame_kind: int = 0              # 0 velocity, 1 displacement, 2 acceleration, 3 all three


class Plan:
    """A set of scenarios advanced together on one GPU (owns the C plan)."""

    def __init__(self, scenarios, run: RunConfig, precision: int = 64, path: int = 0,
                 steps_per_graph: int = 0, tile_elems: int = 0, device: int = 0, rows_per_block: int = 0):
        self.lib = native.load()
        self.scenarios = list(scenarios)
        self.run = run
        self._keep = []  # arrays referenced by the C structs during creation
        n = len(self.scenarios)
        meshes = (native.ShmMesh * n)()
        mats = (native.ShmMaterial * n)()
        runs = (native.ShmRun * n)()
        for i, sc in enumerate(self.scenarios):
            self._fill(sc, meshes[i], mats[i], runs[i])
        opt = native.ShmOptions(precision, path, steps_per_graph, tile_elems, device, rows_per_block)
        handle = C.c_void_p()
        st = self.lib.shm_plan_create(n, meshes, mats, runs, C.byref(opt), C.byref(handle))
        self.handle = handle
        if st != native.SHM_OK:
            msg = self.lib.shm_last_error(handle).decode() if handle.value else ""
            self.lib.shm_plan_destroy(handle)
            self.handle = None
            raise native.ShmError(st, msg)
        self._keep.clear()
        self._refresh_info()
        self.nscen = n
        self.nft = run.nft
        self.nf = 5

    def _refresh_info(self):
        info = (C.c_int64 * 10)()
        self.lib.shm_plan_info(self.handle, info)
        self.info = dict(nnode=info[0], fen=info[1], ndof=info[2], path=info[3], precision=info[4],
                         nframes=info[5], launches_per_step=info[6], tile=info[7], rows_per_block=info[8],
                         nfields=info[9], persistent=info[3] == 2 and info[6] == 0)

    def autotune(self, steps: int = 20):
        """Pick the structured kernel's lane-group width, rows per task and
        launch mode (per-step launches or one persistent launch) by timing."""
        t, r, ms = C.c_int32(), C.c_int32(), C.c_float()
        self._check(self.lib.shm_autotune(self.handle, int(steps), C.byref(t), C.byref(r), C.byref(ms)))
        self._refresh_info()
        return dict(tile=t.value, rows_per_block=r.value, persistent=self.info["persistent"],
                    ms_per_step=ms.value)

    def forward_backward(self, target, signals=None, ckpt_every: int = 200):
        """Misfit J (per scenario) and dJ/dd_e (d_e = 1 - elem_keep) by the
        discrete adjoint with checkpoints every ``ckpt_every`` steps.
        ``target`` is a list of [nft, n_out] arrays (one per scenario)."""
        st = np.ascontiguousarray(self.signals() if signals is None else signals, dtype=np.float64)
        tgt = np.concatenate([np.asarray(t, float).T.reshape(-1) for t in target]) if len(target) else np.zeros(1)
        mis = np.zeros(self.nscen)
        grad = np.zeros(self.info["fen"])
        self._check(self.lib.shm_forward_backward(self.handle, native.ptr(st), native.ptr(tgt), native.ptr(mis),
                                                  native.ptr(grad), int(ckpt_every), None))
        out, e0 = [], 0
        for sc in self.scenarios:
            fen = np.asarray(sc.mesh["nodes"]).shape[0]
            out.append(grad[e0:e0 + fen].copy())
            e0 += fen
        return mis, out

    def set_persistent(self, enable: bool = True, spin_limit: int = -1):
        """Advance in one cooperative launch per call, the CTAs meeting at a
        device-wide barrier between steps (FP32 plans on the structured fused
        kernel).  ``spin_limit`` bounds each barrier wait in polls (< 0: the
        default); a wait that runs out raises SHM_ERR_TIMEOUT."""
        self._check(self.lib.shm_set_persistent(self.handle, int(bool(enable)), int(spin_limit)))
        self._refresh_info()

    def set_frame_staging(self, values: int):
        """Values per staging buffer of the frame readback (default 4 M)."""
        self._check(self.lib.shm_set_frame_staging(self.handle, int(values)))

    def set_guard_interval(self, steps: int):
        """Blow-up guard every ``steps`` time steps besides the frame steps
        (0: at frame steps only, as the reference)."""
        self._check(self.lib.shm_set_guard_interval(self.handle, int(steps)))

    def set_adjoint_store(self, max_bytes: int | str | None = None) -> int:
        """Bytes forward_backward may keep for the last segments' states:
        None = half of the device's free memory (the default), "spare" = the
        free memory less 8 GiB, 0 = recompute every segment.  Returns the
        number of segments the previous call kept."""
        n = C.c_int32()
        code = -3 if max_bytes is None else (-1 if max_bytes == "spare" else int(max_bytes))
        self._check(self.lib.shm_set_adjoint_store(self.handle, code, C.byref(n)))
        return n.value

    def stored_segments(self) -> int:
        n = C.c_int32()
        self._check(self.lib.shm_set_adjoint_store(self.handle, -2, C.byref(n)))
        return n.value

    def forward_backward_timing(self) -> dict:
        """Device ms of the last forward_backward's forward pass, segment
        recomputes and adjoint steps."""
        ms = (C.c_float * 3)()
        self._check(self.lib.shm_forward_backward_timing(self.handle, ms))
        return dict(forward_ms=ms[0], recompute_ms=ms[1], adjoint_ms=ms[2])

    def _arr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self._keep.append(a)
        return a

    def _fill(self, sc: Scenario, m, mt, r):
        mesh = sc.mesh
        nodes = self._arr(np.asarray(mesh["nodes"]).T, np.int32)   # column-major [fen x npe]
        coords = self._arr(np.asarray(mesh["coords"], float).T, np.float64)
        fen, npe = np.asarray(mesh["nodes"]).shape
        m.fen, m.npe, m.nnode = fen, npe, np.asarray(mesh["coords"]).shape[0]
        m.nodes = native.ptr(nodes, native.I32P)
        m.coords = native.ptr(coords)
        if mesh.get("I_G") is not None:
            IG = self._arr(np.asarray(mesh["I_G"]).T, np.int32)
            IL = self._arr(np.asarray(mesh["I_L"]).T, np.int32)
            m.basket_rows = np.asarray(mesh["I_G"]).shape[0]
            m.I_G, m.I_L = native.ptr(IG, native.I32P), native.ptr(IL, native.I32P)
        else:
            m.basket_rows = 0
        m.grid_nex = int(mesh.get("nex", 0)) if mesh.get("structured", True) else 0
        m.grid_ney = int(mesh.get("ney", 0)) if mesh.get("structured", True) else 0
        tab = self._arr(np.atleast_2d(sc.mat_table), np.float64)
        mt.nmat = tab.shape[0]
        mt.table = native.ptr(tab)
        mt.elem_mat = native.ptr(self._arr(sc.elem_mat, np.int32), native.I32P) if sc.elem_mat is not None else None
        mt.elem_keep = native.ptr(self._arr(sc.elem_keep, np.float64)) if sc.elem_keep is not None else None
        run = self.run
        r.dt, r.nft, r.nn_first = run.dt, run.nft, run.nn_first
        r.eta_xy, r.eta_z = run.eta_xy, run.eta_z
        fd = self._arr(sc.force_dof, np.int32)
        fv = self._arr(sc.force_val, np.float64)
        r.n_force, r.force_dof, r.force_val = len(fd), native.ptr(fd, native.I32P), native.ptr(fv)
        od = self._arr(sc.out_dof, np.int32)
        r.n_out, r.out_dof = len(od), native.ptr(od, native.I32P)
        if sc.sensors:
            ptrs = np.zeros(len(sc.sensors) + 1, np.int32)
            ptrs[1:] = np.cumsum([len(s) for s in sc.sensors])
            els = np.concatenate([np.asarray(s, np.int32) for s in sc.sensors])
            r.n_sens = len(sc.sensors)
            r.sens_ptr = native.ptr(self._arr(ptrs, np.int32), native.I32P)
            r.sens_el = native.ptr(self._arr(els, np.int32), native.I32P)
            p = sc.pzt
            r.pzt_thickness, r.g33, r.e31, r.e32 = p["pzt_thickness"], p["g33"], p["e31"], p["e32"]
        else:
            r.n_sens = 0
        r.h = run.h
        r.frm_int, r.frame_dof, r.frame_kind = run.frm_int, run.frame_dof, run.frame_kind
        if sc.pressure is not None:
            pt = self._arr(sc.pressure["times"], np.float64)
            pn = self._arr(np.asarray(sc.pressure["nodal"], float).reshape(len(pt), -1), np.float64)
            r.n_pframes, r.p_times, r.p_nodal = len(pt), native.ptr(pt), native.ptr(pn)
        else:
            r.n_pframes = 0

    # ------------------------------------------------------------------
    def _check(self, st):
        native.check(self.lib, self.handle, st)

    def close(self):
        if self.handle is not None:
            self.lib.shm_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def signals(self):
        return np.stack([np.asarray(sc.signal, float) for sc in self.scenarios])

    def forward(self, signals=None, want_frames=False):
        """Whole MAIN LOOP for every scenario; returns per-scenario outputs."""
        st = np.ascontiguousarray(self.signals() if signals is None else signals, dtype=np.float64)
        nout = sum(len(s.out_dof) for s in self.scenarios)
        nsens = sum(len(s.sensors) for s in self.scenarios)
        displ = np.zeros(max(nout, 1) * self.nft)
        volt = np.zeros(max(nsens, 1) * self.nft)
        nfr = self.info["nframes"]
        frames = (np.zeros(max(nfr * self.info["nfields"] * self.info["nnode"], 1))
                  if (want_frames and nfr) else None)
        self._check(self.lib.shm_forward(self.handle, native.ptr(st), native.ptr(displ), native.ptr(volt),
                                         native.ptr(frames), None))
        return self._split(displ, volt, frames)

    def _split(self, displ, volt, frames):
        out = []
        o = s_ = fo = 0
        for sc in self.scenarios:
            no, ns = len(sc.out_dof), len(sc.sensors)
            nnode = np.asarray(sc.mesh["coords"]).shape[0]
            # [nft, n] views of the library's [n][nft] arrays (the MATLAB layout)
            d = displ[o * self.nft:(o + no) * self.nft].reshape(no, self.nft).T
            v = volt[s_ * self.nft:(s_ + ns) * self.nft].reshape(ns, self.nft).T
            res = dict(displ=d, voltage=v)
            if frames is not None:
                nfr, nfl = self.info["nframes"], self.info["nfields"]
                # a view: the scenarios' frames are disjoint slices of one array
                res["frames"] = frames[fo:fo + nfr * nfl * nnode].reshape(nfr, nfl, nnode)
                fo += nfr * nfl * nnode
            out.append(res)
            o += no
            s_ += ns
        return out

    def reset(self):
        self._check(self.lib.shm_reset(self.handle))

    def set_signal(self, signals=None):
        st = np.ascontiguousarray(self.signals() if signals is None else signals, dtype=np.float64)
        self._check(self.lib.shm_set_signal(self.handle, native.ptr(st), None))

    def advance(self, nsteps):
        self._check(self.lib.shm_advance(self.handle, int(nsteps), None))

    def time_steps(self, nsteps) -> float:
        ms = C.c_float()
        self._check(self.lib.shm_time_steps(self.handle, int(nsteps), C.byref(ms)))
        return ms.value

    def read_outputs(self, want_frames=False):
        nout = sum(len(s.out_dof) for s in self.scenarios)
        nsens = sum(len(s.sensors) for s in self.scenarios)
        displ = np.zeros(max(nout, 1) * self.nft)
        volt = np.zeros(max(nsens, 1) * self.nft)
        nfr = self.info["nframes"]
        frames = (np.zeros(max(nfr * self.info["nfields"] * self.info["nnode"], 1))
                  if (want_frames and nfr) else None)
        self._check(self.lib.shm_read_outputs(self.handle, native.ptr(displ), native.ptr(volt),
                                              native.ptr(frames), None))
        return self._split(displ, volt, frames)

    def get_state(self):
        n = self.info["nnode"]
        U = np.zeros(self.nf * n)
        Uo = np.zeros(self.nf * n)
        self._check(self.lib.shm_get_state(self.handle, native.ptr(U), native.ptr(Uo)))
        return U, Uo

    def set_state(self, U, Uold, nn):
        U = np.ascontiguousarray(U, np.float64)
        Uo = np.ascontiguousarray(Uold, np.float64)
        self._check(self.lib.shm_set_state(self.handle, native.ptr(U), native.ptr(Uo), int(nn)))

    def apply_stiffness(self, U):
        U = np.ascontiguousarray(U, np.float64)
        F = np.zeros_like(U)
        self._check(self.lib.shm_apply_stiffness(self.handle, native.ptr(U), native.ptr(F)))
        return F

    def mass(self):
        mg = np.zeros(self.nf * self.info["nnode"])
        self._check(self.lib.shm_mass(self.handle, native.ptr(mg)))
        return mg


@dataclass
class SolidScenario:
    """One laminate modelled with 3D solid elements (6x6x3 nodes, 3 DOF/node)."""
    mesh: dict                        # nodes [fen,108] 1-based, coords [nnode,3]
    mat_table: np.ndarray             # [nmat, 14] (materials.solid_row)
    elem_mat: np.ndarray | None = None
    elem_keep: np.ndarray | None = None
    force_dof: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))   # 3*(node-1)+{1,2,3}
    force_val: np.ndarray = field(default_factory=lambda: np.zeros(0))
    out_dof: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    signal: np.ndarray | None = None
    sensors: list = field(default_factory=list)


class SolidPlan(Plan):
    """3D-solid scenarios on one GPU (shm_solid_plan_create)."""

    def __init__(self, scenarios, run: RunConfig, precision: int = 64, steps_per_graph: int = 0, device: int = 0):
        self.lib = native.load()
        self.scenarios = list(scenarios)
        self.run = run
        self._keep = []
        n = len(self.scenarios)
        meshes = (native.ShmSolidMesh * n)()
        mats = (native.ShmSolidMaterial * n)()
        runs = (native.ShmRun * n)()
        for i, sc in enumerate(self.scenarios):
            m, mt, r = meshes[i], mats[i], runs[i]
            nodes = self._arr(np.asarray(sc.mesh["nodes"]).T, np.int32)
            coords = self._arr(np.asarray(sc.mesh["coords"], float).T, np.float64)
            m.fen, m.npe = np.asarray(sc.mesh["nodes"]).shape
            m.nnode = np.asarray(sc.mesh["coords"]).shape[0]
            m.nodes, m.coords = native.ptr(nodes, native.I32P), native.ptr(coords)
            m.basket_rows = 0
            tab = self._arr(np.atleast_2d(sc.mat_table), np.float64)
            mt.nmat, mt.table = tab.shape[0], native.ptr(tab)
            mt.elem_mat = native.ptr(self._arr(sc.elem_mat, np.int32), native.I32P) if sc.elem_mat is not None \
                else None
            mt.elem_keep = native.ptr(self._arr(sc.elem_keep, np.float64)) if sc.elem_keep is not None else None
            r.dt, r.nft, r.nn_first = run.dt, run.nft, run.nn_first
            r.eta_xy, r.eta_z = run.eta_xy, run.eta_z
            fd, fv = self._arr(sc.force_dof, np.int32), self._arr(sc.force_val, np.float64)
            r.n_force, r.force_dof, r.force_val = len(fd), native.ptr(fd, native.I32P), native.ptr(fv)
            od = self._arr(sc.out_dof, np.int32)
            r.n_out, r.out_dof = len(od), native.ptr(od, native.I32P)
            r.n_sens = 0
            r.h = run.h
            r.frm_int, r.frame_dof, r.frame_kind = run.frm_int, run.frame_dof, run.frame_kind
        opt = native.ShmOptions(precision, 1, steps_per_graph, 0, device, 0)
        handle = C.c_void_p()
        st = self.lib.shm_solid_plan_create(n, meshes, mats, runs, C.byref(opt), C.byref(handle))
        self.handle = handle
        if st != native.SHM_OK:
            msg = self.lib.shm_last_error(handle).decode() if handle.value else ""
            self.lib.shm_plan_destroy(handle)
            self.handle = None
            raise native.ShmError(st, msg)
        self._keep.clear()
        self._refresh_info()
        self.nscen = n
        self.nft = run.nft
        self.nf = 3


# ----------------------------------------------------------------------
# the reference's entry point
# ----------------------------------------------------------------------

def hanning_signal(dt, nft, f_1, f_2, t_1=0.0):
    """Hann-windowed tone burst (Hanning_signal.m:12-23): returns t, st."""
    t = np.arange(nft) * dt
    t_2 = t_1 + 1.0 / f_1
    on = (t >= t_1) & (t <= t_2)
    st = np.where(on, 0.5 * (1 - np.cos(2 * np.pi * f_1 * (t - t_2))) * np.sin(2 * np.pi * f_2 * (t - t_1)), 0.0)
    return t, st


def random_signal(nft: int, seed: int = 0) -> np.ndarray:
    """White-noise excitation st ~ N(0, 1) of length nft
    (main_flat_shell_multi_pzt_c_random_exc_signals.m:137-139 draws it with
    MATLAB's randn; the stream here is numpy's, seeded)."""
    return np.random.default_rng(seed).standard_normal(nft)


def _laminate(inputs):
    """Laminate of an input file: a material table row (``mat_table``, with
    ply thicknesses ``lh``) or the ply constants q11..q66, rho, lh, lalpha of
    the _c variants (composite_plate_c_delam_pzt.m).  Returns (laminate dict
    or None, table [nmat, 23], total thickness h)."""
    from . import materials as M
    if "mat_table" in inputs:
        return None, np.atleast_2d(inputs["mat_table"]), float(np.sum(inputs["lh"]))
    q = {k: inputs[k] for k in ("q11", "q12", "q22", "q44", "q55", "q66")}
    lam = M.laminate(q, inputs["rho"], inputs["lh"], inputs["lalpha"])
    return lam, table_row(lam)[None, :], lam["h"]


def _pzt_elements(mesh):
    """PZT element lists of a mesh file, 0-based: ``pztEl`` as a cell array
    (a list of 1-based element vectors, main_flat_shell_multi_pzt_c.m:47-50)
    or as a matrix with one PZT per row (main_flat_shell.m:128-136)."""
    pe = mesh.get("pztEl")
    if pe is None:
        return []
    if isinstance(pe, np.ndarray) and pe.dtype != object and pe.ndim == 2:
        rows = [r for r in pe]
    elif isinstance(pe, np.ndarray) and pe.dtype != object:
        rows = [pe] if pe.size else []
    else:
        rows = list(pe)
    return [np.asarray(r, np.int64).ravel() - 1 for r in rows if np.asarray(r).size]


def _pzt_plate(inputs, mesh, lam, h, pzt_elems, actuator):
    """Bonded PZTs (all elements of every PZT carry the piezo layer,
    composite_plate_c_delam_pzt.m) and the equivalent loads of PZT
    ``actuator`` driven at V0 (main_flat_shell.m:144-225).  Returns
    (table, elem_mat, force_dof, force_val, pzt constants)."""
    from . import materials as M
    from . import pzt as PZ
    if lam is None:
        raise ValueError("PZT plates need the ply constants q11..q66, rho, lh, lalpha (not a material table)")
    pm = M.pzt_material(np.asarray(inputs["Spzt"], float), np.asarray(inputs["dp"], float),
                        np.asarray(inputs["epsT"], float), float(inputs.get("theta_pzt", 0.0)))
    t_pzt = float(inputs["pzt_thickness"])
    lam_p = M.add_piezo_layer(lam, pm["Qpzt"], float(inputs["rho_pzt"]), t_pzt)
    fen = np.asarray(mesh["nodes"]).shape[0]
    elem_mat = np.zeros(fen, np.int32)
    for e in pzt_elems:
        elem_mat[e] = 1
    Fa = PZ.actuator_loads(mesh, pzt_elems[actuator], t_pzt, h, float(inputs["V0"]), pm["epzt"], pm["gpzt"])
    nzi = np.nonzero(Fa)[0]
    table = np.stack([table_row(lam), table_row(lam_p)])
    pzt = dict(pzt_thickness=t_pzt, g33=pm["g33"], e31=pm["e31"], e32=pm["e32"])
    return table, elem_mat, (nzi + 1).astype(np.int32), Fa[nzi], pzt


def _frame_interval(inputs, nft):
    """frm_int of the input file: floor(nft/nFrames) for an even nft, the
    input's own frm_int for an odd one (main_flat_shell_multi_pzt_c.m:37-43)."""
    nframes = int(inputs.get("nFrames", 0))
    if not nframes:
        return 0, 0
    if nft % 2 and "frm_int" in inputs:
        return nframes, int(inputs["frm_int"])
    return nframes, nft // nframes


def _solve_and_write(sc, run, test_case, output_name, precision, t, nframes, fv, total_nodes, with_voltage):
    """Runs the plan and writes the reference's files: displ<N>.mat,
    voltage<N>.mat (PZT sensors), time<N>.mat (minTime, averageTime,
    TotalNofNodes, t) and the frame files; returns t_frames."""
    from scipy.io import savemat
    os.makedirs(output_name, exist_ok=True)
    nft, frm_int, nn_first = run.nft, run.frm_int, run.nn_first
    tic = time.perf_counter()
    plan = Plan([sc], run, precision=precision)
    try:
        res = plan.forward(want_frames=frm_int > 0)[0]
    finally:
        plan.close()
    elapsed = time.perf_counter() - tic
    if with_voltage:
        savemat(os.path.join(output_name, f"voltage{test_case}.mat"), {"voltage": res["voltage"]})
    savemat(os.path.join(output_name, f"displ{test_case}.mat"), {"displ": res["displ"]})
    # minTime is the fastest step in the reference (tic/toc per step); the
    # engine runs the loop as one device job, so both are the mean step time
    savemat(os.path.join(output_name, f"time{test_case}.mat"),
            {"minTime": elapsed / max(nft - 1, 1), "averageTime": elapsed / max(nft - 1, 1),
             "TotalNofNodes": total_nodes, "t": t})
    t_frames = np.zeros(nframes)
    if "frames" in res:
        names = [p + c for p in {"displacement": "U", "velocity": "V", "acceleration": "A",
                                 "all": "UVA"}[fv] for c in ("x", "Fix", "y", "Fiy", "z")]
        first = (nn_first + frm_int - 1) // frm_int
        for c in range(min(res["frames"].shape[0], nframes)):
            t_frames[c] = t[(c + first) * frm_int - 1]
            for name, fld in zip(names, res["frames"][c]):
                savemat(os.path.join(output_name, f"{name}_frame{c + 1}.mat"), {name: fld[:, None]})
    return t_frames


_KINDS = {"velocity": 0, "displacement": 1, "acceleration": 2, "all": 3}


def main_flat_shell(test_case, inputs: dict, mesh: dict, mode: str = "gpu", output_name: str = ".",
                    tasks=(), precision: int = 64, variant: str = "main_flat_shell"):
    """Flat-shell forward solve with the reference's interface and outputs.

    inputs: the fields of an ``inputs/input<N>.m`` script (nft, tt, f_1, f_2,
    t_1, nFrames, field_variable, etad_xy, etad_z, V0, and the laminate as a
    material table ``mat_table`` with ``lh`` or q11..q66 + rho + lh + lalpha;
    for a PZT plate also Spzt, dp, epsT, theta_pzt, rho_pzt, pzt_thickness).
    mesh:   the fields of the mesh .mat file (nodes, coords, optional I_G, I_L,
    mesh_min, mesh_max, nex/ney for structured plates, pztEl).
    variant: 'main_flat_shell' (dt = tt/nft, loop nn = 2..nft, output and
    force at the node nearest (mesh_max - mesh_min)/2; with ``pztEl`` the
    first PZT is actuator and sensor instead of the point force,
    main_flat_shell.m:121-225) or 'force_excit_c' (dt = tt/(nft-1),
    nn = 1..nft, force at ``force_coords``, outputs at ``output_coords``).
    Writes displ<test_case>.mat, voltage<test_case>.mat (PZT plates,
    main_flat_shell.m:925), time<test_case>.mat with TotalNofNodes = dof/3 as
    main_flat_shell.m:929 computes it (the 'force_excit_c' variant: dof/5)
    and the wavefield frames {U,V,A}{x,Fix,y,Fiy,z}_frame<c>.mat of
    field_variable 'displacement', 'velocity', 'acceleration' or 'all'
    (main_flat_shell.m:806-885) into output_name; returns t_frames.
    """
    if mode != "gpu":
        raise ValueError("this engine runs the time loop on the GPU only (mode='gpu')")
    from . import mesh as MS

    nft = int(inputs["nft"])
    if variant == "main_flat_shell":
        dt, nn_first = inputs["tt"] / nft, 2
    else:
        dt, nn_first = inputs["tt"] / (nft - 1), 1
    t, st = hanning_signal(dt, nft, inputs["f_1"], inputs["f_2"], inputs.get("t_1", 0.0))
    lam, table, h = _laminate(inputs)
    coords = np.asarray(mesh["coords"], float)
    if variant == "main_flat_shell":
        cen = (np.asarray(mesh["mesh_max"]) - np.asarray(mesh["mesh_min"])) / 2
        out_nodes = [MS.nearest_node(coords, cen[0], cen[1])]
        force_node = out_nodes[0]
    else:
        out_nodes = [MS.nearest_node(coords, x, y) for x, y in np.atleast_2d(inputs["output_coords"])]
        fc = np.atleast_2d(inputs["force_coords"])[0]
        force_node = MS.nearest_node(coords, fc[0], fc[1])
    nframes = int(inputs.get("nFrames", 0))
    frm_int = nft // nframes if nframes else 0
    fv = inputs.get("field_variable", "velocity")
    if fv not in _KINDS:
        raise ValueError(f"field_variable must be one of {sorted(_KINDS)}")
    pzts = _pzt_elements(mesh) if variant == "main_flat_shell" else []
    if pzts:
        table, elem_mat, fdof, fval, pzt = _pzt_plate(inputs, mesh, lam, h, pzts[:1], 0)
        sc = Scenario(mesh=mesh, mat_table=table, elem_mat=elem_mat, force_dof=fdof, force_val=fval,
                      out_dof=5 * np.array(out_nodes, np.int32), signal=st, sensors=[pzts[0]], pzt=pzt)
    else:
        sc = Scenario(mesh=mesh, mat_table=table, force_dof=np.array([5 * force_node], np.int32),
                      force_val=np.array([inputs["V0"]]), out_dof=5 * np.array(out_nodes, np.int32), signal=st)
    run = RunConfig(dt=dt, nft=nft, nn_first=nn_first, eta_xy=inputs.get("etad_xy", 0.0),
                    eta_z=inputs.get("etad_z", 0.0), h=h, frm_int=frm_int, frame_dof=0, frame_kind=_KINDS[fv])
    dof = 5 * coords.shape[0]
    total = dof / 3 if variant == "main_flat_shell" else dof / 5
    return _solve_and_write(sc, run, test_case, output_name, precision, t, nframes, fv, total, bool(pzts))


def main_flat_shell_multi_pzt_c(actuator_no, test_case, inputs: dict, mesh: dict, mode: str = "gpu",
                                output_name: str = ".", tasks=(), precision: int = 64):
    """The reference's benchmarked solver entry point
    ``t_frames = main_flat_shell_multi_pzt_c(actuator_no, test_case, input_no,
    meshfile, mode, output_name, tasks)``
    (src/models/flat_shell/flat_shell_engine/main_flat_shell_multi_pzt_c.m:1).

    Every PZT of the mesh (``pztEl``: a list of 1-based element vectors) is
    bonded (piezo layer in its elements, composite_plate_c_delam_pzt.m) and
    is a sensor; PZT ``actuator_no`` (1-based) is driven at V0 by the Hann
    burst (:150-230).  dt = tt/(nft-1), loop nn = 1..nft (:154,577); the
    output is w at the node nearest (mesh_max - mesh_min)/2 (:57-60).
    Writes voltage<test_case>.mat [nft x nPZT], displ<test_case>.mat,
    time<test_case>.mat with TotalNofNodes = dof/5 (:860-861) and the frame
    files of field_variable (:696-835) into output_name; returns t_frames.
    inputs as for ``main_flat_shell`` (ply constants and PZT constants
    required)."""
    if mode != "gpu":
        raise ValueError("this engine runs the time loop on the GPU only (mode='gpu')")
    from . import mesh as MS

    nft = int(inputs["nft"])
    dt = inputs["tt"] / (nft - 1)
    t, st = hanning_signal(dt, nft, inputs["f_1"], inputs["f_2"], inputs.get("t_1", 0.0))
    lam, _, h = _laminate(inputs)
    pzts = _pzt_elements(mesh)
    if not 1 <= int(actuator_no) <= len(pzts):
        raise ValueError(f"actuator_no must be 1..{len(pzts)} (the mesh's pztEl)")
    table, elem_mat, fdof, fval, pzt = _pzt_plate(inputs, mesh, lam, h, pzts, int(actuator_no) - 1)
    coords = np.asarray(mesh["coords"], float)
    cen = (np.asarray(mesh["mesh_max"]) - np.asarray(mesh["mesh_min"])) / 2
    out_node = MS.nearest_node(coords, cen[0], cen[1])
    nframes, frm_int = _frame_interval(inputs, nft)
    fv = inputs.get("field_variable", "velocity")
    if fv not in _KINDS:
        raise ValueError(f"field_variable must be one of {sorted(_KINDS)}")
    sc = Scenario(mesh=mesh, mat_table=table, elem_mat=elem_mat, force_dof=fdof, force_val=fval,
                  out_dof=np.array([5 * out_node], np.int32), signal=st, sensors=pzts, pzt=pzt)
    run = RunConfig(dt=dt, nft=nft, nn_first=1, eta_xy=inputs.get("etad_xy", 0.0),
                    eta_z=inputs.get("etad_z", 0.0), h=h, frm_int=frm_int, frame_dof=0, frame_kind=_KINDS[fv])
    dof = 5 * coords.shape[0]
    return _solve_and_write(sc, run, test_case, output_name, precision, t, nframes, fv, dof / 5, True)
