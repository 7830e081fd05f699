"""tinyfluids_gb300: the tinyfluids time step on GB300 (sm_103a).

A drop-in for the reference's hot path, ``tinyfluids.jax_tinyfluids``:
``fluid`` (conversions, CFL dt, the split HLL step) and ``time_integration``
(the run-to-time loop), with the same names, arguments and [5, nx, ny, nz]
float32 layout, on CUDA tensors.  All compute runs in the hand-written kernels
of ``csrc/`` behind the C ABI in ``include/tinyfluids_gb300.h``.
"""
from . import fluid, time_integration, initial_conditions, diagnostics  # noqa: F401
from .fluid import (DENSITY_INDEX, PRESSURE_INDEX, VAR_AXIS, VELOCITY_X_INDEX,  # noqa: F401
                    VELOCITY_Y_INDEX, VELOCITY_Z_INDEX, X_AXIS, Y_AXIS, Z_AXIS,
                    _cfl_time_step, _euler_flux, _evolve_state, _evolve_state_along_axis,
                    _hll_solver, _open_boundaries, conserved_state_from_primitive,
                    exact_arithmetic, get_max_wave_speeds, get_wave_speeds,
                    primitive_state_from_conserved, resolved_tile, set_exact,
                    speed_of_sound)
from .initial_conditions import overpressure, setup_ics, shear_layer  # noqa: F401
from .time_integration import (host_runs_workspace_bytes, run_steps, step,  # noqa: F401
                               time_integration_host)
from .time_integration import time_integration as time_integration_fn  # noqa: F401
from ._lib import TinyfluidsError, library_path  # noqa: F401

__version__ = "0.1.0"
