"""ctypes binding of the C-ABI library ``_lib/libtinyfluids_gb300.so``.

The library is the only compute path of this package: there is no CPU or
PyTorch fallback.  If it is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_LOCK = threading.Lock()
_LIB = None
_LIB_CHECKED = None

c_int = ctypes.c_int
c_uint = ctypes.c_uint
c_float = ctypes.c_float
c_ll = ctypes.c_longlong
c_ull = ctypes.c_ulonglong
vp = ctypes.c_void_p
c_char_p = ctypes.c_char_p


class TileConfig(ctypes.Structure):
    """tf_tile_config: tile rows (8, 16, 32), x planes per CTA, plane loader
    (0 auto, 1 per-thread loads, 2 TMA-staged)."""
    _fields_ = [("rows", c_int), ("lx", c_int), ("loader", c_int)]


class Instance(ctypes.Structure):
    """tf_instance: one member of a batch."""
    _fields_ = [("W_in", vp), ("W_out", vp), ("work", vp), ("ctl", vp),
                ("nx", c_int), ("ny", c_int), ("nz", c_int), ("flags", c_uint),
                ("dx", c_float), ("gamma", c_float), ("cfl", c_float), ("t_final", c_float),
                ("fixed_dt", c_float), ("max_steps", c_int), ("lx", c_int),
                ("reserved", c_int)]


class BatchConfig(ctypes.Structure):
    """tf_batch_config."""
    _fields_ = [("rows", c_int), ("exact", c_int), ("persistent", c_int),
                ("ctas_per_sm", c_int), ("wait_limit", c_ull)]


# name -> (restype, argtypes); mirrors include/tinyfluids_gb300.h
SIGNATURES = {
    "tf_abi_version": (c_int, []),
    "tf_status_string": (c_char_p, [c_int]),
    "tf_last_error": (c_char_p, []),
    "tf_ctl_bytes": (c_ull, []),
    "tf_conserved_from_primitive": (c_int, [vp, vp, c_ll, c_float, vp]),
    "tf_primitive_from_conserved": (c_int, [vp, vp, c_ll, c_float, vp]),
    "tf_cfl_time_step": (c_int, [vp, c_int, c_int, c_int, c_float, c_float, c_float, vp, vp]),
    "tf_evolve_state": (c_int, [vp, vp, c_int, c_int, c_int, c_float, c_float, vp, c_float,
                                c_uint, vp, vp]),
    "tf_evolve_state_diag": (c_int, [vp, vp, c_int, c_int, c_int, c_float, c_float, vp,
                                     c_float, c_uint, vp, vp, vp, c_int, vp]),
    "tf_diagnostics": (c_int, [vp, c_int, c_int, c_int, c_float, vp, vp, c_int, vp]),
    "tf_resolve_tile": (c_int, [c_int, c_int, c_int, c_uint, vp, vp]),
    "tf_debug_checked": (c_int, []),
    "tf_debug_set_graph_loop_cap": (c_int, [c_int]),
    "tf_debug_set_loop_start_time": (c_int, [c_float]),
    "tf_debug_force_64bit_offsets": (c_int, [c_int]),
    "tf_debug_reset": (c_int, [vp, c_ll]),
    "tf_debug_oob_count": (c_ll, []),
    "tf_debug_adjoint_sweep_per_cell": (c_int, [vp, vp, vp, c_int, c_int, c_int, c_float,
                                                c_float, c_float, c_int, vp]),
    "tf_time_integration": (c_int, [vp, vp, vp, vp, c_int, c_int, c_int, c_float, c_float,
                                    c_float, c_float, c_int, c_float, c_uint, vp, vp, vp]),
    "tf_evolve_along_axis": (c_int, [vp, vp, c_int, c_int, c_int, c_float, c_float, vp,
                                     c_float, c_int, c_uint, vp]),
    "tf_time_integration_noalloc": (c_int, [vp, vp, c_int, c_int, c_int, c_float, c_float,
                                            c_float, c_float, c_int, c_float, c_uint, vp, vp]),
    "tf_host_runs_workspace_bytes": (c_ull, [c_int, c_int, c_int, c_int]),
    "tf_time_integration_host": (c_int, [vp, vp, c_int, c_int, c_int, c_int, c_float, c_float,
                                         c_float, c_float, c_int, c_float, c_uint, vp, vp, c_ull,
                                         vp, vp]),
    "tf_batch_workspace_bytes": (c_ull, [c_int]),
    "tf_batch_prepare": (c_int, [vp, c_int, vp, vp, c_ull, vp]),
    "tf_batch_run": (c_int, [vp, c_int, c_int, vp]),
    "tf_batch_error": (c_int, [vp, vp, vp]),
    "tf_batch_release": (c_int, [vp]),
    "tf_speed_of_sound": (c_int, [vp, vp, vp, c_ll, c_float, vp]),
    "tf_euler_flux": (c_int, [vp, vp, c_ll, c_float, c_int, vp]),
    "tf_wave_speeds": (c_int, [vp, vp, vp, vp, c_ll, c_float, c_int, vp]),
    "tf_max_wave_speeds": (c_int, [vp, vp, c_ll, c_float, c_int, vp, vp]),
    "tf_hll_flux": (c_int, [vp, vp, vp, c_ll, c_float, c_int, vp]),
    "tf_open_boundaries": (c_int, [vp, vp, c_int, c_int, c_int, c_int, c_uint, c_uint, vp]),
    "tf_adjoint_sweep": (c_int, [vp, vp, vp, c_int, c_int, c_int, c_float, c_float, c_float,
                                 c_int, vp]),
    "tf_adjoint_sweep_f64": (c_int, [vp, vp, vp, c_int, c_int, c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, c_int, vp]),
    "tf_sweep_conserved_f64": (c_int, [vp, vp, c_int, c_int, c_int, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, c_int, vp]),
    "tf_ics_injection_cube": (c_int, [vp, c_int, c_int, vp]),
    "tf_ics_overpressure": (c_int, [vp, c_int, c_ull, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]),
    "tf_ics_shear_layer": (c_int, [vp, c_int, c_ull, ctypes.c_double, vp]),
}

TF_OK = 0
TF_FLAG_OPEN_BOUNDARIES = 1
TF_FLAG_EXACT = 2
TF_FLAG_IN_CONSERVED = 4
TF_FLAG_OUT_CONSERVED = 8
TF_FLAG_HOST_LOOP = 16


class TinyfluidsError(RuntimeError):
    """A C-ABI call returned a non-zero tf_status."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


def library_path() -> str:
    return _build.LIB


def load():
    """Load (once) and return the C-ABI library; raises if it was not built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(
                f"tinyfluids_gb300 CUDA library not found at {path}; build it with "
                "`python -m tinyfluids_gb300.build` (nvcc, sm_103a). There is no CPU fallback.")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if L.tf_abi_version() != 1:
            raise RuntimeError("tinyfluids_gb300 library ABI mismatch")
        _LIB = L
    return _LIB


def load_checked():
    """The checked build of the library (TF_CHECKED=1: range-checked accesses
    and per-cell write counts), built on first use into its own file.  A
    separate handle: the product library stays the one ``call`` uses."""
    global _LIB_CHECKED
    with _LOCK:
        if _LIB_CHECKED is None:
            path = _build.build(checked=True)
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            if L.tf_debug_checked() != 1:
                raise RuntimeError("the checked library was not built with TF_CHECKED=1")
            _LIB_CHECKED = L
    return _LIB_CHECKED


def call(name, *args):
    """Call a C-ABI function and raise TinyfluidsError on a non-zero status."""
    L = load()
    st = getattr(L, name)(*args)
    if st != TF_OK:
        msg = L.tf_last_error().decode(errors="replace")
        raise TinyfluidsError(st, f"{name}: {L.tf_status_string(st).decode()}: {msg}")
    return st
