"""Drop-in for ``tinyfluids.jax_tinyfluids.fluid`` on a GB300.

Same function names, positional arguments and ``[5, nx, ny, nz]`` float32
layout as the reference (fluid.py:10-578).  States are CUDA ``torch.Tensor``s;
every function enqueues hand-written sm_103a kernels through the C ABI of
``include/tinyfluids_gb300.h`` on the tensor's current stream and returns new
tensors (inputs are never modified, like the reference's functional arrays).

Arithmetic.  By default the step uses the fast policy (conserved state
between sweeps, FMAs, one reciprocal per cell and per interface): it agrees
with the reference's float32 results to the tolerance stated in the tests.
``set_exact(True)`` (or ``exact=True``) selects the reference's own op order,
which is bit-identical to the float32 oracle.
"""
from __future__ import annotations

import contextlib
import ctypes

import torch

from . import _lib

# fluid.py:14-22
DENSITY_INDEX = 0
VELOCITY_X_INDEX = 1
VELOCITY_Y_INDEX = 2
VELOCITY_Z_INDEX = 3
PRESSURE_INDEX = 4
VAR_AXIS = 0
X_AXIS = 1
Y_AXIS = 2
Z_AXIS = 3

_EXACT = False


def set_exact(flag: bool) -> None:
    """Select the reference op order (True) or the fast arithmetic (False) globally."""
    global _EXACT
    _EXACT = bool(flag)


def is_exact() -> bool:
    return _EXACT


@contextlib.contextmanager
def exact_arithmetic(flag: bool = True):
    """Context manager form of :func:`set_exact`."""
    old = _EXACT
    set_exact(flag)
    try:
        yield
    finally:
        set_exact(old)


def _flags(handle_boundaries: bool, exact) -> int:
    ex = _EXACT if exact is None else bool(exact)
    return ((_lib.TF_FLAG_OPEN_BOUNDARIES if handle_boundaries else 0)
            | (_lib.TF_FLAG_EXACT if ex else 0))


def check_state(state, name="primitive_state") -> torch.Tensor:
    """Validate a [5, nx, ny, nz] float32 CUDA state (the reference's STATE_TYPE,
    fluid.py:10, checked by jaxtyping/beartype) and return it contiguous."""
    if not isinstance(state, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor, got {type(state).__name__}")
    if state.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {state.dtype}")
    if state.dim() != 4 or state.shape[0] != 5:
        raise TypeError(f"{name} must have shape [5, nx, ny, nz], got {tuple(state.shape)}")
    if not state.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (this package has no CPU path)")
    if min(state.shape[1:]) < 1:
        raise ValueError(f"{name} has an empty axis: {tuple(state.shape)}")
    return state.contiguous()


def _scalar(x, name) -> float:
    if isinstance(x, torch.Tensor):
        if x.numel() != 1:
            raise TypeError(f"{name} must be a scalar")
        return float(x.item())
    return float(x)


def _stream(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def _dt_args(dt, device):
    """(dt_host, dt_dev pointer, keep-alive) for a float or a 0-d CUDA tensor."""
    if isinstance(dt, torch.Tensor):
        if dt.numel() != 1:
            raise TypeError("dt must be a scalar")
        if dt.is_cuda:
            d = dt.reshape(()).to(device=device, dtype=torch.float32).contiguous()
            return 0.0, d.data_ptr(), d
        return float(dt.item()), None, None
    return float(dt), None, None


def new_ctl(device) -> torch.Tensor:
    """A zeroed device control block (tf_ctl, 64 bytes) as 16 int32."""
    return torch.zeros(16, dtype=torch.int32, device=device)


# ctl field offsets (int32 words), include/tinyfluids_gb300.h tf_ctl
CTL_T, CTL_DT, CTL_TFINAL, CTL_CFLDX, CTL_WS, CTL_DONE, CTL_ITER, CTL_ACTIVE, \
    CTL_MAXSTEPS, CTL_STATUS, CTL_MAXSPEED = range(11)


# ---------------------------------------------------------------------------
# fluid.py:30-103
# ---------------------------------------------------------------------------
def conserved_state_from_primitive(primitive_state, gamma):
    """fluid.py:30-67: (rho, rho*u, p/(gamma-1) + 0.5*rho*|u|^2)."""
    W = check_state(primitive_state)
    with torch.cuda.device(W.device):
        U = torch.empty_like(W)
        _lib.call("tf_conserved_from_primitive", W.data_ptr(), U.data_ptr(),
                  W[0].numel(), _scalar(gamma, "gamma"), _stream(W))
    return U


def primitive_state_from_conserved(conserved_state, gamma):
    """fluid.py:71-103: (rho, m/rho, (gamma-1)*rho*(E/rho - 0.5*|u|^2))."""
    U = check_state(conserved_state, "conserved_state")
    with torch.cuda.device(U.device):
        W = torch.empty_like(U)
        _lib.call("tf_primitive_from_conserved", U.data_ptr(), W.data_ptr(),
                  U[0].numel(), _scalar(gamma, "gamma"), _stream(U))
    return W


# ---------------------------------------------------------------------------
# fluid.py:105-413 -- the reference's building blocks (reference op order)
# ---------------------------------------------------------------------------
def _field(x, name):
    if not isinstance(x, torch.Tensor) or x.dtype != torch.float32 or not x.is_cuda:
        raise TypeError(f"{name} must be a float32 CUDA tensor")
    return x.contiguous()


def _pair(left, right):
    L = check_state(left, "primitives_left")
    R = check_state(right, "primitives_right")
    if L.shape != R.shape or L.device != R.device:
        raise TypeError("primitives_left and primitives_right must match")
    return L, R


def _vel(i):
    i = int(i)
    if i not in (VELOCITY_X_INDEX, VELOCITY_Y_INDEX, VELOCITY_Z_INDEX):
        raise ValueError("flux_direction_index must be 1, 2 or 3")
    return i


def speed_of_sound(rho, p, gamma):
    """fluid.py:106-117: sqrt(gamma*p/rho) elementwise."""
    rho, p = _field(rho, "rho"), _field(p, "p")
    if rho.shape != p.shape:
        raise TypeError("rho and p must have the same shape")
    with torch.cuda.device(rho.device):
        c = torch.empty_like(rho)
        _lib.call("tf_speed_of_sound", rho.data_ptr(), p.data_ptr(), c.data_ptr(), rho.numel(),
                  _scalar(gamma, "gamma"), _stream(rho))
    return c


def get_wave_speeds(primitives_left, primitives_right, gamma, flux_direction_index):
    """fluid.py:121-160: (S-, S+) = (min(uL-cL, uR-cR, 0), max(uL+cL, uR+cR, 0))."""
    L, R = _pair(primitives_left, primitives_right)
    with torch.cuda.device(L.device):
        sm = torch.empty_like(L[0])
        sp = torch.empty_like(L[0])
        _lib.call("tf_wave_speeds", L.data_ptr(), R.data_ptr(), sm.data_ptr(), sp.data_ptr(),
                  L[0].numel(), _scalar(gamma, "gamma"), _vel(flux_direction_index), _stream(L))
    return sm, sp


def get_max_wave_speeds(primitives_left, primitives_right, gamma, flux_direction_index):
    """fluid.py:164-195: max(max|S+|, max|S-|) as a 0-d CUDA tensor."""
    L, R = _pair(primitives_left, primitives_right)
    with torch.cuda.device(L.device):
        ctl = new_ctl(L.device)
        _lib.call("tf_max_wave_speeds", L.data_ptr(), R.data_ptr(), L[0].numel(),
                  _scalar(gamma, "gamma"), _vel(flux_direction_index), ctl.data_ptr(), _stream(L))
    return ctl.view(torch.float32)[CTL_MAXSPEED].clone()


def _euler_flux(primitive_state, gamma, flux_direction_index):
    """fluid.py:208-259: the physical flux along the given velocity index."""
    W = check_state(primitive_state)
    with torch.cuda.device(W.device):
        F = torch.empty_like(W)
        _lib.call("tf_euler_flux", W.data_ptr(), F.data_ptr(), W[0].numel(),
                  _scalar(gamma, "gamma"), _vel(flux_direction_index), _stream(W))
    return F


def _hll_solver(primitives_left, primitives_right, gamma, flux_direction_index):
    """fluid.py:263-305: the HLL flux of every (left, right) pair."""
    L, R = _pair(primitives_left, primitives_right)
    with torch.cuda.device(L.device):
        F = torch.empty_like(L)
        _lib.call("tf_hll_flux", L.data_ptr(), R.data_ptr(), F.data_ptr(), L[0].numel(),
                  _scalar(gamma, "gamma"), _vel(flux_direction_index), _stream(L))
    return F


def _open_boundary_call(W, num_ghost_cells, lo, hi):
    W = check_state(W)
    _, nx, ny, nz = W.shape
    with torch.cuda.device(W.device):
        out = torch.empty_like(W)
        _lib.call("tf_open_boundaries", W.data_ptr(), out.data_ptr(), nx, ny, nz,
                  int(num_ghost_cells), lo, hi, _stream(W))
    return out


def _open_boundaries(primitive_state, num_ghost_cells):
    """fluid.py:384-413: zero-gradient ghost cells on every face (x, y, z)."""
    return _open_boundary_call(primitive_state, num_ghost_cells, 7, 7)


def _open_left_boundary(primitive_state, num_ghost_cells, axis):
    """fluid.py:358-379 (axis X_AXIS, Y_AXIS or Z_AXIS)."""
    if axis not in (X_AXIS, Y_AXIS, Z_AXIS):
        raise ValueError("axis must be X_AXIS, Y_AXIS or Z_AXIS")
    return _open_boundary_call(primitive_state, num_ghost_cells, 1 << (axis - 1), 0)


def _open_right_boundary(primitive_state, num_ghost_cells, axis):
    """fluid.py:335-354 (axis X_AXIS, Y_AXIS or Z_AXIS)."""
    if axis not in (X_AXIS, Y_AXIS, Z_AXIS):
        raise ValueError("axis must be X_AXIS, Y_AXIS or Z_AXIS")
    return _open_boundary_call(primitive_state, num_ghost_cells, 0, 1 << (axis - 1))


# ---------------------------------------------------------------------------
# fluid.py:427-504
# ---------------------------------------------------------------------------
def _cfl_time_step(primitive_state, grid_spacing, gamma, C_CFL=0.4):
    """fluid.py:427-504: C_CFL*dx / max wave speed, as a 0-d float32 CUDA tensor.

    The maximum over periodic interfaces of max(|S+|, |S-|) is reduced in its
    per-cell form max_d |v_d| + c, which is equal bit for bit."""
    W = check_state(primitive_state)
    _, nx, ny, nz = W.shape
    with torch.cuda.device(W.device):
        ctl = new_ctl(W.device)
        _lib.call("tf_cfl_time_step", W.data_ptr(), nx, ny, nz, float(grid_spacing),
                  _scalar(gamma, "gamma"), _scalar(C_CFL, "C_CFL"), ctl.data_ptr(), _stream(W))
    return ctl.view(torch.float32)[CTL_DT].clone()


# ---------------------------------------------------------------------------
# fluid.py:508-578
# ---------------------------------------------------------------------------
def _evolve_state(primitive_state, grid_spacing, dt, gamma, handle_boundaries=False, *,
                  exact=None, tile=None, conserved=False):
    """fluid.py:562-578: optional open boundaries, then the x, y, z HLL sweeps,
    fused into one kernel pass.  ``dt`` is a float or a 0-d CUDA tensor (for
    example the result of :func:`_cfl_time_step`).  ``conserved=True`` (fast
    arithmetic, default tile): the state in and out is conserved (rho, m, E),
    equal bit for bit to three ``_evolve_state_along_axis`` sweeps with
    conserved input and output."""
    W = check_state(primitive_state)
    _, nx, ny, nz = W.shape
    flags = _flags(handle_boundaries, exact)
    if conserved:
        flags |= _lib.TF_FLAG_IN_CONSERVED | _lib.TF_FLAG_OUT_CONSERVED
    with torch.cuda.device(W.device):
        out = torch.empty_like(W)
        dt_host, dt_dev, keep = _dt_args(dt, W.device)
        tc = None if conserved and tile is None else _tile_arg(tile, W, exact)
        _lib.call("tf_evolve_state", W.data_ptr(), out.data_ptr(), nx, ny, nz,
                  float(grid_spacing), dt_host, dt_dev, _scalar(gamma, "gamma"),
                  flags, tc, _stream(W))
        del keep
    return out


def _evolve_state_along_axis(primitive_state, grid_spacing, dt, gamma, axis, *,
                             exact=None, open_boundaries=False, conserved_in=False,
                             conserved_out=False):
    """fluid.py:508-557: one periodic HLL sweep along ``axis`` (X_AXIS, Y_AXIS or
    Z_AXIS).  ``open_boundaries`` applies the handle_boundaries remap to the
    input first (the x sweep of an open-boundary step).  With the fast
    arithmetic, ``conserved_in``/``conserved_out`` take/return conserved
    states, so that x (prim->cons), y, z (cons->prim) equal the fused step."""
    W = check_state(primitive_state)
    if axis not in (X_AXIS, Y_AXIS, Z_AXIS):
        raise ValueError("axis must be X_AXIS, Y_AXIS or Z_AXIS")
    _, nx, ny, nz = W.shape
    with torch.cuda.device(W.device):
        out = torch.empty_like(W)
        dt_host, dt_dev, keep = _dt_args(dt, W.device)
        _lib.call("tf_evolve_along_axis", W.data_ptr(), out.data_ptr(), nx, ny, nz,
                  float(grid_spacing), dt_host, dt_dev, _scalar(gamma, "gamma"), axis - 1,
                  _flags(open_boundaries, exact)
                  | (_lib.TF_FLAG_IN_CONSERVED if conserved_in else 0)
                  | (_lib.TF_FLAG_OUT_CONSERVED if conserved_out else 0), _stream(W))
        del keep
    return out


def resolved_tile(shape, handle_boundaries=False, exact=None, tile=None):
    """The tile a fused step on a grid of `shape` (nx, ny, nz) runs:
    (rows, lx, layout) with layout "ldg" / "tma" (x-marching) or "ym"
    (y-marching) and the chunk length resolved."""
    nx, ny, nz = (int(v) for v in shape)
    out = _lib.TileConfig()
    _lib.call("tf_resolve_tile", nx, ny, nz, _flags(handle_boundaries, exact),
              _tile_arg(tile, None, exact), ctypes.byref(out))
    return out.rows, out.lx, {0: "ldg", 1: "ldg", 2: "tma", 3: "ym"}[out.loader]


def _tile_arg(tile, state=None, exact=None):
    """tf_tile_config for `tile`: None (built-in choice), (rows, lx),
    (rows, lx, loader) with loader "auto" | "ldg" | "tma" (x-marching tile)
    or "ym" (y-marching tile, 8 or 16 rows), or "auto" (the autotuner's
    measured best for this grid shape)."""
    if tile is None:
        return None
    if isinstance(tile, str):
        if tile != "auto" or state is None:
            raise ValueError("tile must be None, (rows, lx) or 'auto'")
        from . import autotune
        ex = _EXACT if exact is None else bool(exact)
        tile = autotune.tuned_tile(tuple(state.shape[1:]), exact=ex, device=state.device)
    rows, lx, *rest = tile
    loader = {"auto": 0, "ldg": 1, "tma": 2, "ym": 3}.get(rest[0], rest[0]) if rest else 0
    return ctypes.byref(_lib.TileConfig(int(rows), int(lx), int(loader)))
