"""Build recipe for the native library ``libshmsem.so`` (sm_103a only).

``nvcc -gencode arch=compute_103a,code=sm_103a`` cross-compiles on a machine
without a GPU; the library is written in-tree to ``ma-shm_gb300/_build/``.
"""
from __future__ import annotations

import os
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libshmsem.so")
SOURCES = [os.path.join(PKG_DIR, "csrc", f) for f in ("shmsem.cu", "static_stiffness.cu", "wavefield.cu")]
HEADERS = [os.path.join(PKG_DIR, "csrc", f) for f in ("shell_element.cuh", "shell_structured.cuh",
                                                       "shell_structured_f32.cuh", "solid_element.cuh",
                                                       "internal.h")] + [
    os.path.join(REPO_DIR, "include", "shmsem.h")]

NVCC_FLAGS = [
    "-std=c++17", "-O3", "-lineinfo",
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-shared",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(s) > t for s in SOURCES + HEADERS + [__file__])


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libshmsem.so if any source is newer than the library: each
    translation unit in its own nvcc process (in parallel), then one link."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tag = ".tmp.%d" % os.getpid()
    compile_flags = [f for f in NVCC_FLAGS if f != "-shared"]
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + tag + ".o")
        cmd = [nvcc(), *compile_flags, "-I", os.path.join(REPO_DIR, "include"), "-c", "-o", obj, src]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        objs.append(obj)
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    errs = []
    for p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errs.append(out)
    try:
        if errs:
            raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
        tmp = LIB_PATH + tag
        cmd = [nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp, *objs]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc link failed:\n" + res.stdout + res.stderr)
        os.replace(tmp, LIB_PATH)
    finally:
        for o in objs:
            if os.path.exists(o):
                os.remove(o)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
