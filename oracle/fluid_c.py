"""ctypes binding of the C oracle (oracle/fluid_ref.c) -- TEST INFRASTRUCTURE ONLY.

Same functions and argument meaning as oracle/fluid_np.py; arrays are NumPy
[5, nx, ny, nz] float32 (reference scheme) or float64 (FP64 oracle).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        L = ctypes.CDLL(path)
        for suf, ct in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
            P = ctypes.POINTER(ct)
            f = getattr(L, f"orc_cfl_time_step_{suf}")
            f.restype = ct
            f.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ct, ct, ct]
            f = getattr(L, f"orc_evolve_state_{suf}")
            f.restype = None
            f.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ct, ct, ct, ctypes.c_int]
            f = getattr(L, f"orc_time_integration_{suf}")
            f.restype = ctypes.c_int
            f.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ct, ct, ct,
                          ctypes.c_int, ct, ct, ctypes.c_int, P, P]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _prep(W):
    W = np.ascontiguousarray(W)
    if W.dtype not in (np.float32, np.float64) or W.ndim != 4 or W.shape[0] != 5:
        raise TypeError("state must be a [5, nx, ny, nz] float32/float64 array")
    suf = "f32" if W.dtype == np.float32 else "f64"
    ct = ctypes.c_float if suf == "f32" else ctypes.c_double
    return W, suf, ct


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return lib().orc_max_threads()


def _cfl_time_step(W, grid_spacing, gamma, C_CFL=0.4):
    W, suf, ct = _prep(W)
    _, nx, ny, nz = W.shape
    f = getattr(lib(), f"orc_cfl_time_step_{suf}")
    r = f(W.ctypes.data_as(ctypes.POINTER(ct)), nx, ny, nz, grid_spacing, gamma, C_CFL)
    return W.dtype.type(r)


def _evolve_state(W, grid_spacing, dt, gamma, handle_boundaries=False):
    W, suf, ct = _prep(W)
    out = W.copy()
    _, nx, ny, nz = W.shape
    f = getattr(lib(), f"orc_evolve_state_{suf}")
    f(out.ctypes.data_as(ctypes.POINTER(ct)), nx, ny, nz, grid_spacing, dt, gamma,
      int(bool(handle_boundaries)))
    return out


def time_integration(W, grid_spacing, t_final, gamma, handle_boundaries=False,
                     C_CFL=0.4, fixed_dt=0.0, max_steps=-1, return_dts=False):
    """Returns (state, num_iterations[, dts, t])."""
    W, suf, ct = _prep(W)
    out = W.copy()
    _, nx, ny, nz = W.shape
    f = getattr(lib(), f"orc_time_integration_{suf}")
    cap = max_steps if max_steps >= 0 else 100000
    dts = np.zeros(cap, dtype=W.dtype)
    t = ct(0)
    it = f(out.ctypes.data_as(ctypes.POINTER(ct)), nx, ny, nz, grid_spacing, t_final,
           gamma, int(bool(handle_boundaries)), C_CFL, fixed_dt, max_steps,
           dts.ctypes.data_as(ctypes.POINTER(ct)), ctypes.byref(t))
    if return_dts:
        return out, it, dts[:it], W.dtype.type(t.value)
    return out, it


def run_steps(W, grid_spacing, gamma, num_steps, handle_boundaries=False, C_CFL=0.4,
              dt=None):
    """``num_steps`` steps (CFL dt, or the fixed ``dt``); returns (state, dts)."""
    out, it, dts, _ = time_integration(W, grid_spacing, float("inf"), gamma,
                                       handle_boundaries, C_CFL,
                                       0.0 if dt is None else dt, num_steps, True)
    return out, dts
