"""ctypes binding of ``libshmsem.so`` (include/shmsem.h).

This is the test and Python caller of the C ABI; a MATLAB MEX gateway binds the
same entry points.  Loading fails loudly when the library is missing: there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

SHM_OK, SHM_ERR_BAD_ARG, SHM_ERR_CUDA, SHM_ERR_DIVERGED, SHM_ERR_TIMEOUT, SHM_ERR_OOM, SHM_ERR_STATE, \
    SHM_ERR_UNSUPPORTED = range(8)
STATUS_NAMES = {0: "OK", 1: "BAD_ARG", 2: "CUDA", 3: "DIVERGED", 4: "TIMEOUT", 5: "OOM", 6: "STATE",
                7: "UNSUPPORTED"}
SHM_STATIC_MAX_ELEMS = 4096   # element cap of shm_stiffness_static (include/shmsem.h)

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)


class ShmMesh(C.Structure):
    _fields_ = [("fen", C.c_int32), ("npe", C.c_int32), ("nnode", C.c_int32),
                ("nodes", I32P), ("coords", F64P), ("basket_rows", C.c_int32),
                ("I_G", I32P), ("I_L", I32P), ("grid_nex", C.c_int32), ("grid_ney", C.c_int32)]


class ShmMaterial(C.Structure):
    _fields_ = [("nmat", C.c_int32), ("table", F64P), ("elem_mat", I32P), ("elem_keep", F64P)]


class ShmRun(C.Structure):
    _fields_ = [("dt", C.c_double), ("nft", C.c_int32), ("nn_first", C.c_int32),
                ("eta_xy", C.c_double), ("eta_z", C.c_double),
                ("n_force", C.c_int32), ("force_dof", I32P), ("force_val", F64P),
                ("n_out", C.c_int32), ("out_dof", I32P),
                ("n_sens", C.c_int32), ("sens_ptr", I32P), ("sens_el", I32P),
                ("pzt_thickness", C.c_double), ("g33", C.c_double), ("e31", C.c_double),
                ("e32", C.c_double), ("h", C.c_double),
                ("frm_int", C.c_int32), ("frame_dof", C.c_int32), ("frame_kind", C.c_int32),
                ("n_pframes", C.c_int32), ("p_times", F64P), ("p_nodal", F64P)]


class ShmSolidMesh(C.Structure):
    _fields_ = [("fen", C.c_int32), ("npe", C.c_int32), ("nnode", C.c_int32), ("nodes", I32P), ("coords", F64P),
                ("basket_rows", C.c_int32), ("I_G", I32P), ("I_L", I32P)]


class ShmSolidMaterial(C.Structure):
    _fields_ = [("nmat", C.c_int32), ("table", F64P), ("elem_mat", I32P), ("elem_keep", F64P)]


class ShmOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("path", C.c_int32), ("steps_per_graph", C.c_int32),
                ("tile_elems", C.c_int32), ("device", C.c_int32), ("rows_per_block", C.c_int32)]


class ShmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"shm status {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_LIB = None

# every entry point declared in include/shmsem.h, with its ctypes signature
SIGNATURES = {
    "shm_plan_create": (C.c_int, [C.c_int32, C.POINTER(ShmMesh), C.POINTER(ShmMaterial), C.POINTER(ShmRun),
                                  C.POINTER(ShmOptions), C.POINTER(C.c_void_p)]),
    "shm_plan_destroy": (C.c_int, [C.c_void_p]),
    "shm_last_error": (C.c_char_p, [C.c_void_p]),
    "shm_forward": (C.c_int, [C.c_void_p, F64P, F64P, F64P, F64P, C.c_void_p]),
    "shm_set_guard_interval": (C.c_int, [C.c_void_p, C.c_int32]),
    "shm_set_persistent": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "shm_set_frame_staging": (C.c_int, [C.c_void_p, C.c_int64]),
    "shm_reset": (C.c_int, [C.c_void_p]),
    "shm_set_signal": (C.c_int, [C.c_void_p, F64P, C.c_void_p]),
    "shm_advance": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "shm_read_outputs": (C.c_int, [C.c_void_p, F64P, F64P, F64P, C.c_void_p]),
    "shm_time_steps": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "shm_get_state": (C.c_int, [C.c_void_p, F64P, F64P]),
    "shm_set_state": (C.c_int, [C.c_void_p, F64P, F64P, C.c_int32]),
    "shm_apply_stiffness": (C.c_int, [C.c_void_p, F64P, F64P]),
    "shm_plan_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "shm_mass": (C.c_int, [C.c_void_p, F64P]),
    "shm_solid_plan_create": (C.c_int, [C.c_int32, C.POINTER(ShmSolidMesh), C.POINTER(ShmSolidMaterial),
                                        C.POINTER(ShmRun), C.POINTER(ShmOptions), C.POINTER(C.c_void_p)]),
    "shm_forward_backward": (C.c_int, [C.c_void_p, F64P, F64P, F64P, F64P, C.c_int32, C.c_void_p]),
    "shm_forward_backward_timing": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "shm_set_adjoint_store": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int32)]),
    "shm_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                               C.POINTER(C.c_float)]),
    "shm_stiffness_static": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "shm_grid_create": (C.c_int, [C.POINTER(ShmMesh), C.c_int32, I32P, C.c_int32, C.c_int32, C.c_int32,
                                  C.POINTER(C.c_void_p)]),
    "shm_grid_destroy": (C.c_int, [C.c_void_p]),
    "shm_grid_last_error": (C.c_char_p, [C.c_void_p]),
    "shm_grid_points": (C.c_int, [C.c_void_p, F64P, F64P, I32P, F64P, F64P, F64P]),
    "shm_grid_interpolate": (C.c_int, [C.c_void_p, F64P, C.c_int32, C.c_int32, I32P, C.c_int32, C.c_int32,
                                       C.c_double, F64P, C.c_void_p]),
    "shm_grid_interpolate_plan": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                            C.c_double, F64P, C.c_void_p]),
    "shm_grid_time": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                C.c_int32, C.POINTER(C.c_float)]),
}


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load libshmsem.so; raise if it is absent (no fallback path exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"native library missing: {path} (run __graft_entry__.build())")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def ptr(a, ctype=F64P):
    if a is None:
        return None
    return a.ctypes.data_as(ctype)


def check(lib, plan, status):
    if status != SHM_OK:
        msg = lib.shm_last_error(plan).decode() if plan else ""
        raise ShmError(status, msg)
