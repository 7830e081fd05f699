"""Builds the CUDA library of this package for sm_103a (GB300).

``build()`` compiles every ``csrc/*.cu`` with nvcc into object files in
parallel and links ``_lib/libtinyfluids_gb300.so``, the C-ABI library that
``tinyfluids_gb300._lib`` loads.  Nothing here is architecture-portable on
purpose: the kernels are written for sm_103a only.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB_NAME = "libtinyfluids_gb300.so"
LIB = os.path.join(OUT_DIR, LIB_NAME)
# the checked build (TF_CHECKED=1): range-checked accesses and per-cell write
# counts for the tests; never loaded by the package itself
LIB_CHECKED = os.path.join(OUT_DIR, "libtinyfluids_gb300_checked.so")
OBJ_DIR_CHECKED = os.path.join(OUT_DIR, "obj_checked")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the tinyfluids_gb300 CUDA library cannot be built")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return (sorted(glob.glob(os.path.join(CSRC, "*"))) +
            sorted(glob.glob(os.path.join(INCLUDE, "*.h"))) + [os.path.abspath(__file__)])


def is_stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=None,
          checked: bool = False) -> str:
    """Compile (if stale) and return the path of the shared library
    (``checked=True``: the TF_CHECKED=1 verification build)."""
    lib = LIB_CHECKED if checked else LIB
    obj_dir = OBJ_DIR_CHECKED if checked else OBJ_DIR
    if not force and not is_stale(lib):
        return lib
    nvcc = _nvcc()
    os.makedirs(obj_dir, exist_ok=True)
    flags = (ARCH + NVCC_FLAGS + ["-I", INCLUDE] + (["-DTF_CHECKED=1"] if checked else [])
             + list(extra_flags or []))

    def compile_one(src):
        obj = os.path.join(obj_dir, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + f".tmp{os.getpid()}"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
