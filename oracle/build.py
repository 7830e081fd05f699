"""Build recipe for the C oracle (oracle/fluid_ref.c) -- TEST INFRASTRUCTURE ONLY.

Compiles ``oracle/_build/libfluid_ref.so`` with gcc.  ``-ffp-contract=off``
keeps every multiply and add separately rounded (gcc contracts to FMA by
default on aarch64), so the float build matches the NumPy oracle bit for bit.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfluid_ref.so")
SOURCES = [os.path.join(HERE, "fluid_ref.c"), os.path.join(HERE, "fluid_ref_impl.h")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        lib_mtime = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= lib_mtime for s in SOURCES):
            return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-fno-math-errno",
           "-o", tmp, os.path.join(HERE, "fluid_ref.c")]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
