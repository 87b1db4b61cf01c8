"""Wavefield frames on a uniform grid (spec2meshgrid_flat_shell.m) through the C ABI.

``Grid`` owns a ``shm_grid``: the owner element and local coordinates of
every point of an Nx x Ny grid (host set-up, FP64) and the device copy the
interpolation kernel reads.  Frames come either from the host (the
reference's ``{U,V,A}*_frame<n>.mat`` files) or straight from a plan's
device-resident frames.  ``spec2meshgrid_flat_shell`` mirrors the
reference's entry point and output file.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import native

KINDS = {"velocity": 0, "displacement": 1, "acceleration": 2}
_PREFIX = {"displacement": "U", "velocity": "V", "acceleration": "A"}
_COMPONENTS = ("x", "Fix", "y", "Fiy", "z")       # DOF order u, phi_x, v, phi_y, w
# components each motion reads (flat_shell_variable_names.m:8-17)
MOTION_NEEDS = {1: ("x",), 2: ("y",), 3: ("z",), 4: ("Fix",), 5: ("Fiy",), 6: ("x", "Fix"), 7: ("y", "Fiy"),
                8: ("x", "Fix", "y", "Fiy"), 9: ("x", "Fix", "y", "Fiy", "z")}


def variable_name(field_variable: str, motion: int) -> str:
    """``flat_shell_variable_names.m``: name of the interpolated quantity."""
    p = _PREFIX[field_variable]
    tail = {1: "x", 2: "y", 3: "z", 4: "Fix", 5: "Fiy", 6: "x_top", 7: "y_top"}
    if motion in tail:
        return p + tail[motion]
    word = {"displacement": "displacements", "velocity": "velocities", "acceleration": "accelerations"}[field_variable]
    return f"{word}_in_plane" if motion == 8 else f"total_{word}"


class Grid:
    """nx x ny grid over a flat-shell mesh; ``surface`` 'top' or 'bottom'.

    A mesh with ``den_under``/``den_above`` (a split delamination) is
    searched over its first fen - |den_above| elements, and 'top' reads the
    upper sub-laminate's copy of every split node, as the reference does.
    ``device=None`` builds the set-up on the host only.
    """

    def __init__(self, mesh: dict, nx: int, ny: int, surface: str = "top", device: int | None = 0):
        if surface not in ("top", "bottom"):
            raise ValueError("surface must be 'top' or 'bottom'")
        self.lib = native.load()
        self.nx, self.ny, self.surface = int(nx), int(ny), surface
        nodes = np.asarray(mesh["nodes"])
        coords = np.asarray(mesh["coords"], float)
        self.nnode = coords.shape[0]
        fen = nodes.shape[0]
        du = np.asarray(mesh.get("den_under", ()), np.int64)
        da = np.asarray(mesh.get("den_above", ()), np.int64)
        self.fen_search = fen - len(da)
        remap = None
        if surface == "top" and len(da):
            remap = np.arange(1, self.nnode + 1, dtype=np.int32)
            remap[nodes[du].reshape(-1) - 1] = nodes[da].reshape(-1)
        nodes_cm = np.ascontiguousarray(nodes.T, np.int32)     # column-major [fen x 36]
        coords_cm = np.ascontiguousarray(coords.T)             # column-major [nnode x 3]
        ms = native.ShmMesh()
        ms.fen, ms.npe, ms.nnode = fen, nodes.shape[1], self.nnode
        ms.nodes, ms.coords = native.ptr(nodes_cm, native.I32P), native.ptr(coords_cm)
        ms.basket_rows, ms.grid_nex, ms.grid_ney = 0, 0, 0
        h = C.c_void_p()
        st = self.lib.shm_grid_create(C.byref(ms), self.fen_search, native.ptr(remap, native.I32P), self.nx, self.ny,
                                      -1 if device is None else int(device), C.byref(h))
        self.handle = h
        if st != native.SHM_OK:
            msg = self.lib.shm_grid_last_error(h).decode() if h.value else "bad argument"
            self.close()
            raise native.ShmError(st, msg)

    def _check(self, st):
        if st != native.SHM_OK:
            raise native.ShmError(st, self.lib.shm_grid_last_error(self.handle).decode())

    def points(self) -> dict:
        n = self.nx * self.ny
        xp, yp, ks, et = (np.zeros(n) for _ in range(4))
        own = np.zeros(n, np.int32)
        err = C.c_double()
        self._check(self.lib.shm_grid_points(self.handle, native.ptr(xp), native.ptr(yp), native.ptr(own, native.I32P),
                                             native.ptr(ks), native.ptr(et), C.byref(err)))
        return dict(xp=xp, yp=yp, owner=own, ksi=ks, eta=et, max_err=err.value)

    def _images(self, flat: np.ndarray, nframes: int) -> np.ndarray:
        # kernel order p = iy + ny*ix  ->  [nframes, ny, nx]
        return flat.reshape(nframes, self.nx, self.ny).transpose(0, 2, 1).copy()

    def interpolate(self, frames: np.ndarray, dof_field, motion: int, h: float) -> np.ndarray:
        """frames [nframes, nfields, nnode] on the host; dof_field[5] = field
        index of u, phi_x, v, phi_y, w (-1 = absent).  Returns [nframes, ny, nx]."""
        fr = np.ascontiguousarray(frames, float)
        if fr.ndim != 3 or fr.shape[2] != self.nnode:
            raise ValueError("frames must be [nframes, nfields, nnode]")
        df = np.ascontiguousarray(dof_field, np.int32)
        out = np.zeros(max(fr.shape[0], 1) * self.nx * self.ny)
        self._check(self.lib.shm_grid_interpolate(self.handle, native.ptr(fr), fr.shape[0], fr.shape[1],
                                                  native.ptr(df, native.I32P), int(motion),
                                                  0 if self.surface == "top" else 1, float(h), native.ptr(out), None))
        return self._images(out[:fr.shape[0] * self.nx * self.ny], fr.shape[0])

    def from_plan(self, plan, motion: int, h: float, field_variable: str = "velocity", scen: int = 0) -> np.ndarray:
        """Interpolate the device-resident frames of a plan's scenario."""
        nfr = plan.info["nframes"]
        out = np.zeros(max(nfr, 1) * self.nx * self.ny)
        self._check(self.lib.shm_grid_interpolate_plan(self.handle, plan.handle, int(scen), KINDS[field_variable],
                                                       int(motion), 0 if self.surface == "top" else 1, float(h),
                                                       native.ptr(out), None))
        return self._images(out[:nfr * self.nx * self.ny], nfr)

    def time(self, plan, motion: int, h: float, field_variable: str = "velocity", scen: int = 0, reps: int = 5):
        ms = C.c_float()
        self._check(self.lib.shm_grid_time(self.handle, plan.handle, int(scen), KINDS[field_variable], int(motion),
                                           0 if self.surface == "top" else 1, float(h), int(reps), C.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.shm_grid_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def spec2meshgrid_flat_shell(test_case, inputs: dict, mesh: dict, Nx: int, Ny: int, field_variable: str, motion: int,
                             shell_surface: str, input_name: str, output_name: str, device: int = 0) -> np.ndarray:
    """The reference's post-processing entry point (spec2meshgrid_flat_shell.m).

    Reads the frame files ``{U,V,A}<component>_frame<n>.mat`` (n = 1..nFrames)
    of ``field_variable`` that ``motion`` needs from ``input_name``, writes
    ``flat_shell_<variable>_<test_case>_<Nx>x<Ny><surface>.mat`` with
    ``Data`` [Ny, Nx, nFrames] into ``output_name`` and returns Data.
    ``inputs`` carries nFrames and the ply thicknesses lh (h = sum(lh)).
    """
    from scipy.io import loadmat, savemat

    h = float(np.sum(inputs["lh"]))
    nframes = int(inputs["nFrames"])
    prefix = _PREFIX[field_variable]
    comps = MOTION_NEEDS[int(motion)]
    nnode = np.asarray(mesh["coords"]).shape[0]
    frames = np.zeros((nframes, len(comps), nnode))
    for n in range(nframes):
        for k, c in enumerate(comps):
            name = prefix + c
            frames[n, k] = np.asarray(loadmat(os.path.join(input_name, f"{name}_frame{n + 1}.mat"))[name]).reshape(-1)
    dof_field = [comps.index(c) if c in comps else -1 for c in _COMPONENTS]
    g = Grid(mesh, Nx, Ny, shell_surface, device=device)
    try:
        img = g.interpolate(frames, dof_field, motion, h)
    finally:
        g.close()
    data = np.transpose(img, (1, 2, 0))
    os.makedirs(output_name, exist_ok=True)
    fname = f"flat_shell_{variable_name(field_variable, motion)}_{test_case}_{Nx}x{Ny}{shell_surface}.mat"
    savemat(os.path.join(output_name, fname), {"Data": data})
    return data
