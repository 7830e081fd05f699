"""NumPy restatement of the tinyfluids time step -- TEST INFRASTRUCTURE ONLY.

This module is the oracle: a CPU, op-for-op restatement of the reference's
first-order Godunov / HLL Euler step (``tinyfluids/jax_tinyfluids/fluid.py``)
and its run-to-time loop (``tinyfluids/jax_tinyfluids/time_integration.py``).
Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it, and only as the
checker or the timed CPU baseline.  The product path (``tinyfluids_gb300``)
never imports it.

Arithmetic contract.  The reference runs under ``jax.jit`` with x64 off, so
every scalar argument (``gamma``, ``grid_spacing``, ``dt``, ``t_final``,
``C_CFL``) is traced as a float32 value, and every array op is one IEEE
float32 operation.  This file keeps that: scalars are cast to the array dtype
first (``_s``), and each expression keeps the reference's evaluation order
(left-to-right products, ``sqrt(...)**2``, ``(1/dx)*dF*dt``).  NumPy float32
ufuncs round every op separately (no FMA contraction), so with
``dtype=float32`` this is the reference's float32 scheme; with
``dtype=float64`` it is the FP64 oracle of the same scheme.

Parity pin.  The reference ships no field-value tests; its only golden data
are the iteration counts to ``t_final=0.2`` stored in
``results/scaling_data*.npz`` (see ``tests/golden``).  This restatement
reproduces them (``tests/test_oracle.py``).
"""
from __future__ import annotations

import numpy as np

# fluid.py:14-22 -- variable and axis indices of the [5, nx, ny, nz] layout.
DENSITY_INDEX = 0
VELOCITY_X_INDEX = 1
VELOCITY_Y_INDEX = 2
VELOCITY_Z_INDEX = 3
PRESSURE_INDEX = 4
VAR_AXIS = 0
X_AXIS = 1
Y_AXIS = 2
Z_AXIS = 3


def _s(x, dtype):
    """A scalar as the reference sees it under jit: rounded to the array dtype."""
    return np.asarray(x, dtype=np.float64).astype(dtype)[()]


# ----------------------------------------------------------------------------
# fluid.py:28-103 -- primitive <-> conserved
# ----------------------------------------------------------------------------
def conserved_state_from_primitive(primitive_state, gamma):
    """fluid.py:30-67.  E = p/(gamma-1) + 0.5*rho*sqrt(|u|^2)**2, m = rho*u."""
    W = primitive_state
    g = _s(gamma, W.dtype)
    rho = W[DENSITY_INDEX]
    p = W[PRESSURE_INDEX]
    utotal = np.sqrt(W[VELOCITY_X_INDEX] ** 2 + W[VELOCITY_Y_INDEX] ** 2
                     + W[VELOCITY_Z_INDEX] ** 2)
    E = p / (g - 1) + 0.5 * rho * utotal ** 2
    U = W.copy()
    U[PRESSURE_INDEX] = E
    U[VELOCITY_X_INDEX] = rho * W[VELOCITY_X_INDEX]
    U[VELOCITY_Y_INDEX] = rho * W[VELOCITY_Y_INDEX]
    U[VELOCITY_Z_INDEX] = rho * W[VELOCITY_Z_INDEX]
    return U


def primitive_state_from_conserved(conserved_state, gamma):
    """fluid.py:71-103.  u = m/rho, p = (gamma-1)*rho*(E/rho - 0.5*|u|^2)."""
    U = conserved_state
    g = _s(gamma, U.dtype)
    rho = U[DENSITY_INDEX]
    E = U[PRESSURE_INDEX]
    ux = U[VELOCITY_X_INDEX] / rho
    uy = U[VELOCITY_Y_INDEX] / rho
    uz = U[VELOCITY_Z_INDEX] / rho
    u = np.sqrt(ux ** 2 + uy ** 2 + uz ** 2)
    p = (g - 1) * rho * (E / rho - 0.5 * u ** 2)
    W = U.copy()
    W[PRESSURE_INDEX] = p
    W[VELOCITY_X_INDEX] = ux
    W[VELOCITY_Y_INDEX] = uy
    W[VELOCITY_Z_INDEX] = uz
    return W


# ----------------------------------------------------------------------------
# fluid.py:105-195 -- sound speed and HLL wave speeds
# ----------------------------------------------------------------------------
def speed_of_sound(rho, p, gamma):
    """fluid.py:106-117.  c = sqrt(gamma*p/rho)."""
    g = _s(gamma, np.asarray(rho).dtype)
    return np.sqrt(g * p / rho)


def get_wave_speeds(primitives_left, primitives_right, gamma, flux_direction_index):
    """fluid.py:121-160.  S- = min(uL-cL, uR-cR, 0), S+ = max(uL+cL, uR+cR, 0)."""
    rho_L = primitives_left[DENSITY_INDEX]
    u_L = primitives_left[flux_direction_index]
    p_L = primitives_left[PRESSURE_INDEX]
    rho_R = primitives_right[DENSITY_INDEX]
    u_R = primitives_right[flux_direction_index]
    p_R = primitives_right[PRESSURE_INDEX]
    c_L = speed_of_sound(rho_L, p_L, gamma)
    c_R = speed_of_sound(rho_R, p_R, gamma)
    wave_speeds_right_plus = np.maximum(np.maximum(u_L + c_L, u_R + c_R), 0)
    wave_speeds_left_minus = np.minimum(np.minimum(u_L - c_L, u_R - c_R), 0)
    return wave_speeds_left_minus, wave_speeds_right_plus


def get_max_wave_speeds(primitives_left, primitives_right, gamma, flux_direction_index):
    """fluid.py:164-195.  max(max|S+|, max|S-|) over all interfaces."""
    sm, sp = get_wave_speeds(primitives_left, primitives_right, gamma,
                             flux_direction_index)
    return np.maximum(np.max(np.abs(sp)), np.max(np.abs(sm)))


# ----------------------------------------------------------------------------
# fluid.py:206-305 -- Euler flux and HLL interface flux
# ----------------------------------------------------------------------------
def _euler_flux(primitive_state, gamma, flux_direction_index):
    """fluid.py:208-259.  Physical flux along the given velocity index."""
    W = primitive_state
    g = _s(gamma, W.dtype)
    rho = W[DENSITY_INDEX]
    p = W[PRESSURE_INDEX]
    flux_vector = W.copy()
    utotal = np.sqrt(W[VELOCITY_X_INDEX] ** 2 + W[VELOCITY_Y_INDEX] ** 2
                     + W[VELOCITY_Z_INDEX] ** 2)
    E = p / (g - 1) + 0.5 * rho * utotal ** 2
    flux_vector[PRESSURE_INDEX] = flux_vector[PRESSURE_INDEX] + E
    flux_vector[VELOCITY_X_INDEX] = W[VELOCITY_X_INDEX] * rho
    flux_vector[VELOCITY_Y_INDEX] = W[VELOCITY_Y_INDEX] * rho
    flux_vector[VELOCITY_Z_INDEX] = W[VELOCITY_Z_INDEX] * rho
    flux_vector = W[flux_direction_index] * flux_vector
    flux_vector[flux_direction_index] = flux_vector[flux_direction_index] + p
    return flux_vector


def _hll_solver(primitives_left, primitives_right, gamma, flux_direction_index):
    """fluid.py:263-305.  F = (S+ F_L - S- F_R + S- S+ (U_R - U_L)) / (S+ - S-)."""
    fluxes_left = _euler_flux(primitives_left, gamma, flux_direction_index)
    fluxes_right = _euler_flux(primitives_right, gamma, flux_direction_index)
    sm, sp = get_wave_speeds(primitives_left, primitives_right, gamma,
                             flux_direction_index)
    conserved_left = conserved_state_from_primitive(primitives_left, gamma)
    conserved_right = conserved_state_from_primitive(primitives_right, gamma)
    return (sp * fluxes_left - sm * fluxes_right
            + sm * sp * (conserved_right - conserved_left)) / (sp - sm)


# ----------------------------------------------------------------------------
# fluid.py:317-413 -- open (zero-gradient) boundaries
# ----------------------------------------------------------------------------
def _set_along_axis(primitive_state, axis, set_index, get_index):
    """fluid.py:319-331.  state[..., set_index, ...] = state[..., get_index, ...]."""
    W = primitive_state.copy()
    s_set = (slice(None),) * axis + (set_index,)
    s_get = (slice(None),) * axis + (get_index,)
    W[s_set] = W[s_get]
    return W


def _open_right_boundary(primitive_state, num_ghost_cells, axis):
    """fluid.py:335-354."""
    get_index = -num_ghost_cells - 1
    for set_index in range(-num_ghost_cells, 0):
        primitive_state = _set_along_axis(primitive_state, axis, set_index, get_index)
    return primitive_state


def _open_left_boundary(primitive_state, num_ghost_cells, axis):
    """fluid.py:358-379."""
    get_index = num_ghost_cells
    for set_index in range(num_ghost_cells):
        primitive_state = _set_along_axis(primitive_state, axis, set_index, get_index)
    return primitive_state


def _open_boundaries(primitive_state, num_ghost_cells):
    """fluid.py:384-413.  x, then y, then z; left before right on each axis."""
    W = primitive_state
    for axis in (X_AXIS, Y_AXIS, Z_AXIS):
        W = _open_left_boundary(W, num_ghost_cells, axis)
        W = _open_right_boundary(W, num_ghost_cells, axis)
    return W


# ----------------------------------------------------------------------------
# fluid.py:425-578 -- CFL time step and the dimensionally split update
# ----------------------------------------------------------------------------
def _cfl_time_step(primitive_state, grid_spacing, gamma, C_CFL=0.4):
    """fluid.py:427-504.  dt = C_CFL*dx / max over axes and periodic interfaces."""
    W = primitive_state
    dt_ = W.dtype
    maxes = []
    for axis, vel in ((X_AXIS, VELOCITY_X_INDEX), (Y_AXIS, VELOCITY_Y_INDEX),
                      (Z_AXIS, VELOCITY_Z_INDEX)):
        left = np.roll(W, shift=1, axis=axis)
        maxes.append(get_max_wave_speeds(left, W, gamma, vel))
    max_wave_speed = np.maximum(np.maximum(maxes[0], maxes[1]), maxes[2])
    return _s(C_CFL, dt_) * _s(grid_spacing, dt_) / max_wave_speed


def max_wave_speed_per_cell(primitive_state, gamma):
    """max over cells and axes of |u_d| + c.

    Equal, bit for bit in float32, to the interface maximum of fluid.py:457-500
    under periodic wrap: every cell is the right state of its own interface and
    the left state of the next one, c >= 0, and max(u+c, c-u) rounds to |u|+c.
    The CUDA path reduces this per-cell form; ``tests/test_oracle.py`` checks
    the identity against ``_cfl_time_step``.
    """
    W = primitive_state
    c = speed_of_sound(W[DENSITY_INDEX], W[PRESSURE_INDEX], gamma)
    m = np.abs(W[VELOCITY_X_INDEX]) + c
    m = np.maximum(m, np.abs(W[VELOCITY_Y_INDEX]) + c)
    m = np.maximum(m, np.abs(W[VELOCITY_Z_INDEX]) + c)
    return np.max(m)


def _evolve_state_along_axis(primitive_state, grid_spacing, dt, gamma, axis):
    """fluid.py:508-557.  U += (1/dx)*(F_i - F_{i+1})*dt with periodic rolls."""
    W = primitive_state
    d = W.dtype
    conservative_states = conserved_state_from_primitive(W, gamma)
    primitive_state_left = np.roll(W, shift=1, axis=axis)
    fluxes = _hll_solver(primitive_state_left, W, gamma, axis)
    conserved_change = (_s(1, d) / _s(grid_spacing, d)
                        * (fluxes - np.roll(fluxes, shift=-1, axis=axis)) * _s(dt, d))
    conservative_states = conservative_states + conserved_change
    return primitive_state_from_conserved(conservative_states, gamma)


def _evolve_state(primitive_state, grid_spacing, dt, gamma, handle_boundaries=False):
    """fluid.py:562-578.  Optional open BC, then the x, y, z sweeps with one dt."""
    W = primitive_state
    if handle_boundaries:
        W = _open_boundaries(W, 1)
    W = _evolve_state_along_axis(W, grid_spacing, dt, gamma, X_AXIS)
    W = _evolve_state_along_axis(W, grid_spacing, dt, gamma, Y_AXIS)
    W = _evolve_state_along_axis(W, grid_spacing, dt, gamma, Z_AXIS)
    return W


# ----------------------------------------------------------------------------
# time_integration.py:35-128 -- run to t_final
# ----------------------------------------------------------------------------
def time_integration(primitive_state, grid_spacing, t_final, gamma,
                     handle_boundaries=False, shard_mapped=False,
                     padding=None, split=None, C_CFL=0.4, max_steps=None):
    """time_integration.py:94-128 (plain branch) and :63-92 (the while loop).

    ``t`` accumulates in the state's dtype (float32 for the reference), the
    loop test is ``t < t_final`` before each step, and the last step is not
    clamped.  Returns ``(state, num_iterations)``.
    """
    if shard_mapped:
        raise NotImplementedError("shard_map branch is out of scope")
    W = primitive_state
    d = W.dtype
    t = _s(0.0, d)
    tf = _s(t_final, d)
    it = 0
    while t < tf:
        if max_steps is not None and it >= max_steps:
            break
        dt = _cfl_time_step(W, grid_spacing, gamma, C_CFL)
        W = _evolve_state(W, grid_spacing, dt, gamma, handle_boundaries)
        t = (t + dt).astype(d)
        it += 1
    return W, it


def run_steps(primitive_state, grid_spacing, gamma, num_steps,
              handle_boundaries=False, C_CFL=0.4, dt=None):
    """``num_steps`` steps of the same loop body, CFL dt unless ``dt`` is fixed."""
    W = primitive_state
    dts = []
    for _ in range(num_steps):
        step_dt = _cfl_time_step(W, grid_spacing, gamma, C_CFL) if dt is None \
            else _s(dt, W.dtype)
        W = _evolve_state(W, grid_spacing, step_dt, gamma, handle_boundaries)
        dts.append(step_dt)
    return W, np.asarray(dts, dtype=W.dtype)
