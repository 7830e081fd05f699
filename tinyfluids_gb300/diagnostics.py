"""Diagnostics of a state: conserved totals and the density / pressure slice.

The reference inspects a run with ``plot_results`` (scaling_jax.py:75-82),
which shows ``state[DENSITY_INDEX, :, :, n // 2]`` and
``state[PRESSURE_INDEX, :, :, n // 2]`` as images.  Here the same two planes
come back as a ``[2, nx, ny]`` device tensor (and can be written as PGM
images and ``.npy`` arrays, no graphics stack needed), together with the
totals of the conserved variables (rho, rho*vx, rho*vy, rho*vz, E summed over
all cells, the quantities a periodic run conserves).

``step_with_diagnostics`` and ``run_steps_with_diagnostics`` compute them in
the same kernel pass as the (last) step, so a run's final diagnostics cost no
extra read of the state; ``diagnostics`` reads any stored state once.
"""
from __future__ import annotations

import os

import numpy as np
import torch

from . import _lib
from .fluid import CTL_DT, _dt_args, _flags, _scalar, _stream, _tile_arg, check_state
from .time_integration import run_steps

CONSERVED_NAMES = ("mass", "momentum_x", "momentum_y", "momentum_z", "energy")


def _z_slice(z, nz):
    z = nz // 2 if z is None else int(z)
    if not 0 <= z < nz:
        raise ValueError(f"z slice {z} outside [0, {nz})")
    return z


def diagnostics(primitive_state, gamma, z=None, slices=True):
    """(totals, slices) of a primitive state: totals = float64 [5] device
    tensor of the summed conserved variables; slices = float32 [2, nx, ny]
    (rho, p on the plane z, default nz // 2) or None."""
    W = check_state(primitive_state)
    _, nx, ny, nz = W.shape
    zs = _z_slice(z, nz)
    with torch.cuda.device(W.device):
        totals = torch.empty(5, dtype=torch.float64, device=W.device)
        sl = torch.empty((2, nx, ny), dtype=torch.float32, device=W.device) if slices else None
        _lib.call("tf_diagnostics", W.data_ptr(), nx, ny, nz, _scalar(gamma, "gamma"),
                  totals.data_ptr(), sl.data_ptr() if sl is not None else None, zs, _stream(W))
    return totals, sl


def step_with_diagnostics(primitive_state, grid_spacing, dt, gamma, handle_boundaries=False, *,
                          z=None, slices=True, exact=None, tile=None):
    """One ``_evolve_state`` step (same arguments and result) that also returns
    the new state's diagnostics, computed in the same kernel pass:
    (state, totals, slices)."""
    W = check_state(primitive_state)
    _, nx, ny, nz = W.shape
    zs = _z_slice(z, nz)
    with torch.cuda.device(W.device):
        out = torch.empty_like(W)
        totals = torch.empty(5, dtype=torch.float64, device=W.device)
        sl = torch.empty((2, nx, ny), dtype=torch.float32, device=W.device) if slices else None
        dt_host, dt_dev, keep = _dt_args(dt, W.device)
        _lib.call("tf_evolve_state_diag", W.data_ptr(), out.data_ptr(), nx, ny, nz,
                  float(grid_spacing), dt_host, dt_dev, _scalar(gamma, "gamma"),
                  _flags(handle_boundaries, exact), _tile_arg(tile, W, exact),
                  totals.data_ptr(), sl.data_ptr() if sl is not None else None, zs, _stream(W))
        del keep
    return out, totals, sl


def run_steps_with_diagnostics(primitive_state, grid_spacing, gamma, num_steps,
                               handle_boundaries=False, *, C_CFL=0.4, dt=None, z=None,
                               slices=True, exact=None, tile=None):
    """``run_steps`` whose last step also produces the diagnostics of the final
    state in its own pass: (state, totals, slices).  The first num_steps - 1
    steps run in the device loop; the last step takes the dt that loop's final
    epilogue left in the control block (or the fixed ``dt``), so the state is
    bit-identical to ``run_steps`` with the same arguments."""
    n = int(num_steps)
    if n < 1:
        raise ValueError("num_steps must be >= 1")
    W, ctl = run_steps(primitive_state, grid_spacing, gamma, n - 1, handle_boundaries,
                       C_CFL=C_CFL, dt=dt, exact=exact, tile=tile, return_ctl=True)
    if dt is None:
        # tf_ctl.dt: the CFL dt of the next step, read on the device
        last_dt = ctl.view(torch.float32)[CTL_DT:CTL_DT + 1].reshape(())
    else:
        last_dt = float(dt)
    return step_with_diagnostics(W, grid_spacing, last_dt, gamma, handle_boundaries, z=z,
                                 slices=slices, exact=exact, tile=tile)


def integrals(totals, grid_spacing):
    """Totals times the cell volume: the domain integrals of the conserved
    variables (host floats keyed by name)."""
    h = totals.double().cpu().numpy() * float(grid_spacing) ** 3
    return dict(zip(CONSERVED_NAMES, (float(v) for v in h)))


def _write_pgm(path, img):
    a = np.asarray(img, dtype=np.float64)
    lo, hi = float(np.nanmin(a)), float(np.nanmax(a))
    scale = 255.0 / (hi - lo) if hi > lo else 0.0
    g = np.clip(np.nan_to_num((a - lo) * scale), 0, 255).astype(np.uint8)
    # imshow's default orientation of state[:, :, z]: row i = x index i from
    # the top, column j = y index j
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (g.shape[1], g.shape[0]))
        f.write(g.tobytes())


def save_slices(slices, prefix):
    """Writes ``<prefix>_density.pgm`` / ``_pressure.pgm`` (8-bit grayscale,
    min-max scaled) and ``<prefix>_slices.npy`` (the float32 [2, nx, ny]
    array): the headless counterpart of figures/check_N.png.  Returns the
    paths."""
    h = slices.detach().float().cpu().numpy()
    d = os.path.dirname(prefix)
    if d:
        os.makedirs(d, exist_ok=True)
    paths = [f"{prefix}_density.pgm", f"{prefix}_pressure.pgm", f"{prefix}_slices.npy"]
    _write_pgm(paths[0], h[0])
    _write_pgm(paths[1], h[1])
    np.save(paths[2], h)
    return paths
