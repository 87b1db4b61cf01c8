"""The C-ABI library builds, loads and exports every entry point declared in
include/shmsem.h (no compute calls: this file runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "shmsem.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(shm_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("shm_plan_create", "shm_forward", "shm_plan_destroy", "shm_last_error", "shm_advance"):
        assert must in syms


def test_library_exports_declared_symbols(built_pkg):
    lib = ctypes.CDLL(built_pkg.native.lib_path())
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes binding covers exactly the declared ABI
    assert sorted(built_pkg.native.SIGNATURES) == declared_symbols()


def test_library_is_built_for_sm_103a(built_pkg):
    """The build recipe targets sm_103a only (no PTX for other targets)."""
    flags = " ".join(built_pkg.build.NVCC_FLAGS)
    assert "arch=compute_103a,code=sm_103a" in flags
    assert "sm_90" not in flags and "sm_100" not in flags


def test_bad_arguments_fail_without_gpu_work(built_pkg):
    """NULL/invalid arguments are rejected before any device call."""
    lib = built_pkg.native.load()
    h = ctypes.c_void_p()
    st = lib.shm_plan_create(0, None, None, None, None, ctypes.byref(h))
    assert st == built_pkg.native.SHM_ERR_BAD_ARG
    assert lib.shm_plan_destroy(None) == built_pkg.native.SHM_OK


def test_plan_settings_reject_a_null_plan(built_pkg):
    """The plan settings refuse a NULL plan before touching the device."""
    lib = built_pkg.native.load()
    bad = built_pkg.native.SHM_ERR_BAD_ARG
    assert lib.shm_set_persistent(None, 1, -1) == bad
    assert lib.shm_set_frame_staging(None, 1024) == bad
    assert lib.shm_set_guard_interval(None, 100) == bad
    assert lib.shm_set_adjoint_store(None, 0, None) == bad
